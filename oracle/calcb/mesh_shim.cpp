// Test infrastructure (the oracle's checker of B = curl A, not product code).
// Builds the reference example's own voxel mesh with its mesh maker
// (examples/VoxelFEM/MeshMakerFile/MeshMaker.h:52-83), uniform cells of size h:
//   mesh_shim nx ny nz h
// run in a directory D whose parent holds MeshData/; writes
// ../MeshData/{Node,Edge,Element}.vxldata (and ./mesh.vtk) as the example does.
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <iostream>
#include <fstream>
#include <queue>

using namespace std;

#include "../Defines_Mesh.h"
#include "../Defines_Other.h"
#include "SearchTree.h"
#include "Node_Mesh.h"
#include "Edge.h"
#include "Element.h"
#include "Boundary.h"
#include "T_Vector.h"
#include "MeshMaker.h"

int main(int argc, char **argv) {
    if (argc != 5) {
        fprintf(stderr, "usage: mesh_shim nx ny nz h\n");
        return 2;
    }
    const int nx = atoi(argv[1]), ny = atoi(argv[2]), nz = atoi(argv[3]);
    const double h = atof(argv[4]);
    double len1[] = {h, h, h}, len2[] = {h, h, h};
    int change[] = {nx, ny, nz};  // every cell of the fine size
    MeshMaker mesh(nx, ny, nz, len1, len2, change);
    return 0;
}
