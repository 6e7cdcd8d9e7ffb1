// ss_post.cu -- post-processing beside the solver: flux density B = curl A per
// voxel element at its centre, from the edge unknowns of a solution.
//
// Restates Element::calcB / Element::calcRot of the reference's VoxelFEM
// example (examples/VoxelFEM/Element.cpp:116-168) at the element centre
// (pos_rst = 0): the 12 edges in the example's order (x-edges, y-edges,
// z-edges with the sign tables Data_rk / Data_sk / Data_tk), rot of edge i =
// sign / 8 / L_a / L_b with L the element half-widths, B accumulated edge by
// edge as B += A_edge * rot, edges without an unknown (Dirichlet) skipped.
// Products and sums are rounded one by one (no fused multiply-add), the
// arithmetic of the reference's host build.
#include "sparsesolv_gb300.h"
#include "ss_internal.cuh"
#include "ss_solver.cuh"

namespace ssg {

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }

template <typename T>
__device__ __forceinline__ void acc_rot(T &b, T a, double r);
template <>
__device__ __forceinline__ void acc_rot<double>(double &b, double a, double r) {
    b = dadd(b, dmul(a, r));
}
template <>
__device__ __forceinline__ void acc_rot<cplx>(cplx &b, cplx a, double r) {
    b.x = dadd(b.x, dmul(a.x, r));
    b.y = dadd(b.y, dmul(a.y, r));
}

// the example's local edge tables (Element.cpp, calcB)
__constant__ double c_rk[12] = {0, 0, 0, 0, 1, 1, -1, -1, 1, -1, -1, 1};
__constant__ double c_sk[12] = {1, -1, -1, 1, 0, 0, 0, 0, 1, 1, -1, -1};
__constant__ double c_tk[12] = {1, 1, -1, -1, 1, -1, -1, 1, 0, 0, 0, 0};

template <typename T>
__global__ void k_flux_density(int nx, int ny, int nz, double hx, double hy, double hz, const int *ex, const int *ey,
                               const int *ez, const T *A, T *B) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long ne = (long long)nx * ny * nz;
    if (e >= ne) return;
    const int x = (int)(e % nx), y = (int)((e / nx) % ny), z = (int)(e / ((long long)nx * ny));
    const double Lx = hx / 2.0, Ly = hy / 2.0, Lz = hz / 2.0;
    T b0 = Sc<T>::zero(), b1 = Sc<T>::zero(), b2 = Sc<T>::zero();
    for (int i = 0; i < 12; ++i) {
        const double r = c_rk[i], s = c_sk[i], t = c_tk[i];
        // start node of edge i and its unknown
        int cx = x, cy = y, cz = z;
        const int *map;
        double r0, r1, r2;
        if (i < 4) {
            cy += s > 0 ? 1 : 0;
            cz += t > 0 ? 1 : 0;
            map = ex;
            r0 = 0.0;
            r1 = t * 1.0 / 8.0 / Lx / Lz;
            r2 = -s * 1.0 / 8.0 / Lx / Ly;
        } else if (i < 8) {
            cx += r > 0 ? 1 : 0;
            cz += t > 0 ? 1 : 0;
            map = ey;
            r0 = -t * 1.0 / 8.0 / Ly / Lz;
            r1 = 0.0;
            r2 = r * 1.0 / 8.0 / Lx / Ly;
        } else {
            cx += r > 0 ? 1 : 0;
            cy += s > 0 ? 1 : 0;
            map = ez;
            r0 = s * 1.0 / 8.0 / Ly / Lz;
            r1 = -r * 1.0 / 8.0 / Lx / Lz;
            r2 = 0.0;
        }
        const int id = map[cx + (nx + 1) * (cy + (ny + 1) * (long long)cz)];
        if (id < 0) continue;
        const T a = A[id];
        acc_rot(b0, a, r0);
        acc_rot(b1, a, r1);
        acc_rot(b2, a, r2);
    }
    B[3 * e + 0] = b0;
    B[3 * e + 1] = b1;
    B[3 * e + 2] = b2;
}

template <typename T>
static void flux_density(int nx, int ny, int nz, double hx, double hy, double hz, const int *ex, const int *ey,
                         const int *ez, const T *A, T *B, cudaStream_t s) {
    const long long ne = (long long)nx * ny * nz;
    if (ne == 0) return;
    k_flux_density<T><<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(nx, ny, nz, hx, hy, hz, ex, ey, ez, A, B);
    SSG_LAUNCHED();
}

// host wrapper: inputs from host or device, B to host or device
void flux_density_any(Handle &h, int nx, int ny, int nz, double hx, double hy, double hz, const int *ex,
                      const int *ey, const int *ez, int nunk, const void *A, int vt, void *B, bool on_device) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || !(hx > 0.0) || !(hy > 0.0) || !(hz > 0.0) || nunk < 0)
        throw Error{SSG_ERR_ARG, "bad grid"};
    if (vt != SSG_REAL && vt != SSG_COMPLEX) throw Error{SSG_ERR_ARG, "bad value type"};
    const size_t vb = vt == SSG_COMPLEX ? 16 : 8;
    const size_t nn = (size_t)(nx + 1) * (ny + 1) * (nz + 1);
    const size_t ne = (size_t)nx * ny * nz;
    cudaStream_t s = h.stream;
    DBuf dex, dey, dez, dA, dB;
    const int *pex = ex, *pey = ey, *pez = ez;
    const void *pA = A;
    void *pB = B;
    if (!on_device) {
        dex.alloc(sizeof(int) * nn);
        dey.alloc(sizeof(int) * nn);
        dez.alloc(sizeof(int) * nn);
        dA.alloc(vb * ((size_t)nunk + 1));
        dB.alloc(vb * 3 * ne);
        SSG_CUDA(cudaMemcpyAsync(dex.p, ex, sizeof(int) * nn, cudaMemcpyHostToDevice, s));
        SSG_CUDA(cudaMemcpyAsync(dey.p, ey, sizeof(int) * nn, cudaMemcpyHostToDevice, s));
        SSG_CUDA(cudaMemcpyAsync(dez.p, ez, sizeof(int) * nn, cudaMemcpyHostToDevice, s));
        if (nunk) SSG_CUDA(cudaMemcpyAsync(dA.p, A, vb * (size_t)nunk, cudaMemcpyHostToDevice, s));
        pex = dex.as<int>();
        pey = dey.as<int>();
        pez = dez.as<int>();
        pA = dA.p;
        pB = dB.p;
    }
    if (vt == SSG_COMPLEX)
        flux_density<cplx>(nx, ny, nz, hx, hy, hz, pex, pey, pez, (const cplx *)pA, (cplx *)pB, s);
    else
        flux_density<double>(nx, ny, nz, hx, hy, hz, pex, pey, pez, (const double *)pA, (double *)pB, s);
    if (!on_device) SSG_CUDA(cudaMemcpyAsync(B, pB, vb * 3 * ne, cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace ssg
