// Test infrastructure (the oracle's checker of B = curl A, not product code).
// Runs the reference example's Element::calcB (examples/VoxelFEM/Element.cpp:47-90,
// the element-centre flux density) over a mesh written by its mesh maker:
//   calcb_shim MeshDataDir subid.txt A.bin B.bin
// subid.txt: one matrix index per edge of Edge.vxldata, in file order (the
// example's VoxelMesh::setSubIDs assigns them; the test supplies its own
// numbering); A.bin: doubles indexed by those ids; B.bin: per element of
// Element.vxldata, in file order, int32 x, y, z then doubles B[0..5].
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "Edge.h"
#include "Element.h"
#include "Node.h"

static FILE *open_or_die(const std::string &p, const char *mode) {
    FILE *f = fopen(p.c_str(), mode);
    if (!f) {
        fprintf(stderr, "cannot open %s\n", p.c_str());
        exit(2);
    }
    return f;
}

int main(int argc, char **argv) {
    if (argc != 5) {
        fprintf(stderr, "usage: calcb_shim MeshDataDir subid.txt A.bin B.bin\n");
        return 2;
    }
    const std::string dir = argv[1];
    int nn = 0, gx, gy, gz;
    FILE *f = open_or_die(dir + "/Node.vxldata", "r");
    if (fscanf(f, "%d %d %d %d", &nn, &gx, &gy, &gz) != 4) return 3;
    std::vector<Node> nodes(nn);
    for (int i = 0; i < nn; ++i) {
        int id;
        double x, y, z;
        if (fscanf(f, "%d %lf %lf %lf", &id, &x, &y, &z) != 4 || id < 0 || id >= nn) return 3;
        nodes[id].set(id, x, y, z);
    }
    fclose(f);
    int ne = 0;
    f = open_or_die(dir + "/Edge.vxldata", "r");
    if (fscanf(f, "%d", &ne) != 1) return 3;
    std::vector<Edge> edges(ne);
    for (int i = 0; i < ne; ++i) {
        int id, s, e;
        if (fscanf(f, "%d %d %d", &id, &s, &e) != 3 || id < 0 || id >= ne) return 3;
        edges[id].set(s, e);
        edges[id].setID(id);
    }
    fclose(f);
    f = open_or_die(argv[2], "r");
    int amax = -1;
    for (int i = 0; i < ne; ++i) {
        int sid;
        if (fscanf(f, "%d", &sid) != 1) return 3;
        edges[i].setSubID(sid);
        if (sid > amax) amax = sid;
    }
    fclose(f);
    std::vector<double> A(amax + 1, 0.0);
    f = open_or_die(argv[3], "rb");
    if (amax >= 0 && fread(A.data(), sizeof(double), A.size(), f) != A.size()) return 3;
    fclose(f);
    Element::setNodeData(nodes.data());
    Element::setEdgeData(edges.data());
    int nel = 0;
    f = open_or_die(dir + "/Element.vxldata", "r");
    if (fscanf(f, "%d", &nel) != 1) return 3;
    FILE *o = open_or_die(argv[4], "wb");
    std::vector<Element> els(nel);
    for (int i = 0; i < nel; ++i) {
        int id, x, y, z, n[8], e[12];
        if (fscanf(f, "%d %d %d %d", &id, &x, &y, &z) != 4) return 3;
        for (int k = 0; k < 8; ++k)
            if (fscanf(f, "%d", &n[k]) != 1 || n[k] < 0 || n[k] >= nn) return 3;
        for (int k = 0; k < 12; ++k)
            if (fscanf(f, "%d", &e[k]) != 1 || e[k] < 0 || e[k] >= ne) return 3;
        els[i].set(x, y, z, n, e, id);
        double B[6];
        els[i].calcB(B, A.data());
        const int xyz[3] = {x, y, z};
        fwrite(xyz, sizeof(int), 3, o);
        fwrite(B, sizeof(double), 6, o);
    }
    fclose(f);
    fclose(o);
    return 0;
}
