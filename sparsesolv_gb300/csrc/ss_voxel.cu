// ss_voxel.cu -- the voxel edge-element systems assembled on the device,
// straight to CSR in the handle, with their T-method right-hand sides.
//
// The systems are those of the reference's VoxelFEM example
// (examples/VoxelFEM/VoxelMatrix.cpp:118-201: K = sum_e nu_e Ke, plus
// j omega sigma_e Me for eddy currents; :24-114: b = sum_e Ce t_e from the
// current vector potential on the z-edges), on the grid, node order and edge
// numbering of the host generator (sparsesolv_gb300/voxel/voxelgen.c, which
// follows the example's mesh maker). The result is bit-identical to the host
// generator's:
//   * a row is one edge; its entries come from the (at most four) elements
//     holding the edge, taken in ascending element index (the host's loop
//     order), and within an element from local edges 0..11;
//   * a new column is appended, an existing one accumulated: value += nu_e *
//     Ke[k][m] and += (sigma_e omega) * Me[k][m], products and sums rounded one
//     by one (__dmul_rn / __dadd_rn: no fused multiply-add, as the host
//     generator is compiled without contraction);
//   * the row's columns are then sorted; explicit zeros stay in the pattern;
//   * b_r += sum over the element's z-edges m with t_m != 0 of Ce[k][m] t_m,
//     element by element.
// The element matrices come from the host (the generator's own integrals),
// so both paths use the same 432 numbers.
#include "sparsesolv_gb300.h"
#include "ss_internal.cuh"
#include "ss_solver.cuh"

namespace ssg {

constexpr int VX_MAXROW = 33;  // an interior edge couples with 33 edges, itself included

struct VxGrid {
    int nx, ny, nz;
    const int *map[3];  // unknown of the x/y/z edge starting at node x + (nx+1)(y + (ny+1) z), or -1
};

__device__ __forceinline__ long long vx_node(const VxGrid &g, int x, int y, int z) {
    return (long long)x + (long long)(g.nx + 1) * ((long long)y + (long long)(g.ny + 1) * z);
}

// unknowns of the 12 local edges of element (x, y, z): local edge l = 4 d + 2 b + a,
// direction d, offsets a / b along the first / second transverse axis
__device__ void vx_element_ids(const VxGrid &g, int x, int y, int z, int ids[12]) {
#pragma unroll
    for (int l = 0; l < 12; ++l) {
        const int d = l / 4, a = l & 1, b = (l >> 1) & 1;
        int c[3] = {x, y, z};
        c[d == 0 ? 1 : 0] += a;
        c[d == 2 ? 1 : 2] += b;
        ids[l] = g.map[d][vx_node(g, c[0], c[1], c[2])];
    }
}

// edge r: direction and start node, from the maps
__global__ void k_vx_inverse(VxGrid g, long long nn, int n, int *dir, long long *node, int *err) {
    const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (v >= nn) return;
    for (int d = 0; d < 3; ++d) {
        const int r = g.map[d][v];
        if (r < 0) continue;
        if (r >= n) {
            atomicExch(err, ERR_PATTERN);
            continue;
        }
        dir[r] = d;
        node[r] = v;
    }
}

// one thread per row: COUNT writes the row's entry count; otherwise the row's
// sorted columns and values at rp[r], and b[r]
template <bool COUNT, bool CPLX>
__global__ void k_vx_rows(VxGrid g, int n, const int *dir, const long long *node, const double *mats,
                          const double *nu, const double *sig, double omega, const double *tz, const int *rp, int *cnt,
                          int *col, double *val, double *b, int *err) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int d = dir[r];
    const long long v = node[r];
    if (d < 0 || v < 0) {  // an unknown without an edge
        atomicExch(err, ERR_PATTERN);
        if (COUNT) cnt[r] = 0;
        return;
    }
    const int x0 = (int)(v % (g.nx + 1)), y0 = (int)((v / (g.nx + 1)) % (g.ny + 1));
    const int z0 = (int)(v / ((long long)(g.nx + 1) * (g.ny + 1)));
    const int lim[3] = {g.nx, g.ny, g.nz};
    const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
    // the elements holding the edge, ascending by element index
    long long el[4];
    int loc[4], ne = 0;
    for (int bb = 0; bb < 2; ++bb)
        for (int a = 0; a < 2; ++a) {
            int c[3] = {x0, y0, z0};
            c[t1] -= a;
            c[t2] -= bb;
            if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= lim[0] || c[1] >= lim[1] || c[2] >= lim[2]) continue;
            long long e = (long long)c[0] + (long long)g.nx * ((long long)c[1] + (long long)g.ny * c[2]);
            int l = 4 * d + 2 * bb + a, i = ne++;
            while (i > 0 && el[i - 1] > e) {
                el[i] = el[i - 1];
                loc[i] = loc[i - 1];
                --i;
            }
            el[i] = e;
            loc[i] = l;
        }
    int cols[VX_MAXROW];
    double vk[VX_MAXROW], vm[VX_MAXROW];
    int m_cnt = 0;
    double brow = 0.0;
    for (int q = 0; q < ne; ++q) {
        const long long e = el[q];
        const int x = (int)(e % g.nx), y = (int)((e / g.nx) % g.ny), z = (int)(e / ((long long)g.nx * g.ny));
        int ids[12];
        vx_element_ids(g, x, y, z, ids);
        const int k = loc[q];
        const double nue = COUNT ? 0.0 : nu[e];
        const double se = (COUNT || !sig) ? 0.0 : __dmul_rn(sig[e], omega);
        for (int m = 0; m < 12; ++m) {
            const int c = ids[m];
            if (c < 0) continue;
            int pos = -1;
            for (int t = 0; t < m_cnt; ++t)
                if (cols[t] == c) {
                    pos = t;
                    break;
                }
            if (pos < 0) {
                if (m_cnt == VX_MAXROW) {
                    atomicExch(err, ERR_PATTERN);
                    return;
                }
                pos = m_cnt++;
                cols[pos] = c;
                vk[pos] = 0.0;
                vm[pos] = 0.0;
            }
            if (!COUNT) {
                vk[pos] = __dadd_rn(vk[pos], __dmul_rn(nue, mats[k * 12 + m]));
                vm[pos] = __dadd_rn(vm[pos], __dmul_rn(se, mats[144 + k * 12 + m]));
            }
        }
        if (!COUNT && tz) {
            // only the z-directed local edges (8..11) carry T
            double acc = 0.0;
            for (int m = 8; m < 12; ++m) {
                const int a = m & 1, bb = (m >> 1) & 1;
                const double t = tz[(long long)(x + a) + (long long)(g.nx + 1) * ((long long)(y + bb) + (long long)(g.ny + 1) * z)];
                if (t != 0.0) acc = __dadd_rn(acc, __dmul_rn(mats[288 + k * 12 + m], t));
            }
            brow = __dadd_rn(brow, acc);
        }
    }
    if (COUNT) {
        cnt[r] = m_cnt;
        return;
    }
    if (rp[r + 1] - rp[r] != m_cnt) {
        atomicExch(err, ERR_PATTERN);
        return;
    }
    // columns ascending (they are distinct)
    for (int i = 1; i < m_cnt; ++i) {
        const int kc = cols[i];
        const double kk = vk[i], km = vm[i];
        int j = i - 1;
        while (j >= 0 && cols[j] > kc) {
            cols[j + 1] = cols[j];
            vk[j + 1] = vk[j];
            vm[j + 1] = vm[j];
            --j;
        }
        cols[j + 1] = kc;
        vk[j + 1] = kk;
        vm[j + 1] = km;
    }
    const int o = rp[r];
    for (int i = 0; i < m_cnt; ++i) {
        col[o + i] = cols[i];
        if (CPLX) {
            val[2 * (o + i)] = vk[i];
            val[2 * (o + i) + 1] = vm[i];
        } else {
            val[o + i] = vk[i];
        }
    }
    if (b) {
        if (CPLX) {
            b[2 * r] = brow;
            b[2 * r + 1] = 0.0;
        } else {
            b[r] = brow;
        }
    }
}

void voxel_assemble_any(Handle &h, int nx, int ny, int nz, const int *ex, const int *ey, const int *ez, int nunk,
                        const double *Ke, const double *Me, const double *Ce, const double *nu, const double *sig,
                        double omega, const double *tz, int vt, void *b, bool on_device) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || nunk < 0 || !ex || !ey || !ez || !Ke || !Me || !Ce || !nu)
        throw Error{SSG_ERR_ARG, "bad voxel grid arguments"};
    if (vt != SSG_REAL && vt != SSG_COMPLEX) throw Error{SSG_ERR_ARG, "bad value type"};
    const long long nn = (long long)(nx + 1) * (ny + 1) * (nz + 1);
    const long long nel = (long long)nx * ny * nz;
    const long long ntz = (long long)(nx + 1) * (ny + 1) * nz;
    if (nn > (1ll << 31) || (long long)nunk > 3 * nn) throw Error{SSG_ERR_ARG, "voxel grid too large"};
    cudaStream_t s = h.stream;
    const bool cx = vt == SSG_COMPLEX;
    DBuf dmap[3], dnu, dsig, dtz, dmats, ddir, dnode, drp, dcol, dval, db, tmp;
    const int *pmap[3] = {ex, ey, ez};
    const double *pnu = nu, *psig = sig, *ptz = tz;
    auto up = [&](DBuf &d, const void *src, size_t bytes) {
        d.alloc(bytes);
        SSG_CUDA(cudaMemcpyAsync(d.p, src, bytes, cudaMemcpyHostToDevice, s));
    };
    if (!on_device) {
        for (int q = 0; q < 3; ++q) {
            up(dmap[q], pmap[q], sizeof(int) * (size_t)nn);
            pmap[q] = dmap[q].as<int>();
        }
        up(dnu, nu, sizeof(double) * (size_t)nel);
        pnu = dnu.as<double>();
        if (sig) {
            up(dsig, sig, sizeof(double) * (size_t)nel);
            psig = dsig.as<double>();
        }
        if (tz) {
            up(dtz, tz, sizeof(double) * (size_t)ntz);
            ptz = dtz.as<double>();
        }
    }
    dmats.alloc(sizeof(double) * 432);
    SSG_CUDA(cudaMemcpyAsync(dmats.p, Ke, sizeof(double) * 144, cudaMemcpyHostToDevice, s));
    SSG_CUDA(cudaMemcpyAsync(dmats.as<double>() + 144, Me, sizeof(double) * 144, cudaMemcpyHostToDevice, s));
    SSG_CUDA(cudaMemcpyAsync(dmats.as<double>() + 288, Ce, sizeof(double) * 144, cudaMemcpyHostToDevice, s));
    VxGrid g{nx, ny, nz, {pmap[0], pmap[1], pmap[2]}};
    const int n = nunk;
    DBuf derr;  // this assembly's own status word
    derr.alloc(sizeof(int));
    int *err = derr.as<int>();
    SSG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    ddir.alloc(sizeof(int) * ((size_t)n + 1));
    dnode.alloc(sizeof(long long) * ((size_t)n + 1));
    SSG_CUDA(cudaMemsetAsync(ddir.p, 0xFF, sizeof(int) * ((size_t)n + 1), s));
    SSG_CUDA(cudaMemsetAsync(dnode.p, 0xFF, sizeof(long long) * ((size_t)n + 1), s));
    k_vx_inverse<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(g, nn, n, ddir.as<int>(), dnode.as<long long>(), err);
    SSG_LAUNCHED();
    drp.alloc(sizeof(int) * ((size_t)n + 1));
    SSG_CUDA(cudaMemsetAsync(drp.p, 0, sizeof(int) * ((size_t)n + 1), s));
    const unsigned grid = (unsigned)div_up(std::max(n, 1), 128);
    if (n > 0) {
        k_vx_rows<true, false><<<grid, 128, 0, s>>>(g, n, ddir.as<int>(), dnode.as<long long>(), dmats.as<double>(),
                                                    pnu, psig, omega, ptz, nullptr, drp.as<int>(), nullptr, nullptr,
                                                    nullptr, err);
        SSG_LAUNCHED();
    }
    scan_exclusive(drp.as<int>(), n + 1, nullptr, s, tmp);
    int nnz = 0, herr = 0;
    SSG_CUDA(cudaMemcpyAsync(&nnz, drp.as<int>() + n, sizeof(int), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaStreamSynchronize(s));
    if (herr) throw Error{SSG_ERR_ARG, "edge maps inconsistent with the unknown count"};
    const size_t vb = cx ? 16 : 8;
    dcol.alloc(sizeof(int) * ((size_t)nnz + 1));
    dval.alloc(vb * ((size_t)nnz + 1));
    double *pb = nullptr;
    if (b) {
        if (on_device) {
            pb = (double *)b;
        } else {
            db.alloc(vb * ((size_t)n + 1));
            pb = db.as<double>();
        }
    }
    if (n > 0) {
        if (cx)
            k_vx_rows<false, true><<<grid, 128, 0, s>>>(g, n, ddir.as<int>(), dnode.as<long long>(), dmats.as<double>(),
                                                        pnu, psig, omega, ptz, drp.as<int>(), nullptr, dcol.as<int>(),
                                                        dval.as<double>(), pb, err);
        else
            k_vx_rows<false, false><<<grid, 128, 0, s>>>(g, n, ddir.as<int>(), dnode.as<long long>(),
                                                         dmats.as<double>(), pnu, psig, omega, ptz, drp.as<int>(),
                                                         nullptr, dcol.as<int>(), dval.as<double>(), pb, err);
        SSG_LAUNCHED();
    }
    SSG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaStreamSynchronize(s));
    if (herr) throw Error{SSG_ERR_ARG, "edge maps inconsistent with the grid"};
    h.set_matrix(n, nnz, drp.as<int>(), dcol.as<int>(), dval.as<double>(), vt, cudaMemcpyDeviceToDevice);
    if (b && !on_device && n > 0) {
        SSG_CUDA(cudaMemcpyAsync(b, pb, vb * (size_t)n, cudaMemcpyDeviceToHost, s));
        SSG_CUDA(cudaStreamSynchronize(s));
    }
}

}  // namespace ssg
