// ss_batch.cu -- per-instance Krylov kernels and the batch driver.
//
// The per-instance recurrences are those of the single-system kernels
// (ss_spmv_vec.cu), which restate src/MatSolverICCG.cpp:257-318 and
// src/MatSolverMRTR_ICver.cpp:270-360; the convergence set-up restates
// src/MatSolverICCG.cpp:212-237. Only the reductions differ: fixed tiles
// inside one instance, summed in tile order by the last block.
#include <algorithm>
#include <cstring>

#include "ss_batch.cuh"
#include "ss_kdev.cuh"

namespace ssg {

constexpr int BT = 256;

template <int K>
__device__ __forceinline__ void block_partial(double (&v)[K], double *dst) {
    __shared__ double sh[K][BT / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const double w = warp_sum_d(v[k]);
        if (lane == 0) sh[k][wid] = w;
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double w = lane < BT / 32 ? sh[k][lane] : 0.0;
            w = warp_sum_d(w);
            if (lane == 0) dst[k] = w;
        }
    }
    __syncthreads();
}

// true in every thread of the last block to finish its tiles
__device__ __forceinline__ bool last_block(unsigned *counter) {
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (s_last) __threadfence();
    return s_last != 0;
}

// an instance's tile partials, added in tile order; the loads of D tiles are issued
// together before their additions (a large instance has hundreds of tiles, and one
// L2 round trip per tile dominated the reduction)
template <int K>
__device__ __forceinline__ void inst_sum(const BDev &B, int s, double (&tot)[K]) {
    constexpr int D = K <= 2 ? 16 : 4;
#pragma unroll
    for (int k = 0; k < K; ++k) tot[k] = 0.0;
    const int t1 = B.sys_tile[s + 1];
    for (int t = B.sys_tile[s]; t < t1; t += D) {
        double v[D][K];
#pragma unroll
        for (int u = 0; u < D; ++u)
#pragma unroll
            for (int k = 0; k < K; ++k) v[u][k] = t + u < t1 ? __ldcg(B.part + (size_t)(t + u) * BATCH_PARTS + k) : 0.0;
#pragma unroll
        for (int u = 0; u < D; ++u)
            if (t + u < t1)
#pragma unroll
                for (int k = 0; k < K; ++k) tot[k] += v[u][k];
    }
}

// last block, after the per-instance updates: the batch stays active while any instance is
__device__ __forceinline__ void finish(const BDev &B) {
    int any = 0;
    for (int s = threadIdx.x; s < B.S; s += BT) any |= B.st[s].active;
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) {
        B.ctl->active = any;
        *B.counter = 0u;
    }
}

__device__ __forceinline__ double *inst_log(const BDev &B, int s) { return B.logs + (size_t)s * B.log_stride; }

// ---------------------------------------------------------------- set-up
// |b| per instance (x0 = 0, so r0 = b) and the convergence set-up of
// src/MatSolverICCG.cpp:212-237 (identical in the MRTR solvers)
template <typename T>
__global__ void __launch_bounds__(BT) k_bsetup(BDev B, const T *b) {
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        const int2 tr = B.tile[t];
        double acc[1] = {0.0};
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) acc[0] += Sc<T>::abs2(b[i]);
        block_partial<1>(acc, B.part + (size_t)t * BATCH_PARTS);
    }
    if (!last_block(B.counter)) return;
    for (int s = threadIdx.x; s < B.S; s += BT) {
        KState *st = B.st + s;
        double tot[1];
        inst_sum<1>(B, s, tot);
        const double normB = sqrt(tot[0]), pure = normB;
        double *log = inst_log(B, s);
        st->it = 0;
        if (normB <= 1.0e-30 && pure <= 1.0e-20) {
            st->active = 0;
            st->status = ST_CONVERGED;
            st->log_len = 1;
            log[0] = 0.0;
            continue;
        }
        const double abs_conv = normB * st->conv_cri * 0.9 < 1.0e-20 ? 1.0e-20 : normB * st->conv_cri * 0.9;
        if (pure / normB < st->conv_cri * 0.5 || pure < abs_conv * 0.5) {
            st->active = 0;
            st->status = ST_CONVERGED;
            st->log_len = 0;
            continue;
        }
        st->abs_conv_cri = abs_conv;
        st->normalizer = normB;
        st->log_len = -1;
        log[0] = pure / normB;
        if (st->max_ite <= 0) {
            st->active = 0;
            st->status = ST_MAXIT;
        }
    }
    finish(B);
}

// ICCG set-up: rur0 = r . z
template <typename T>
__global__ void __launch_bounds__(BT) k_brur0(BDev B, const T *r, const T *z) {
    if (!B.ctl->active) return;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        if (!B.act[(size_t)B.tile_sys[t] * B.act_stride]) continue;
        const int2 tr = B.tile[t];
        double acc[2] = {0.0, 0.0};
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) acc_parts<T>(acc, r[i] * z[i]);
        block_partial<2>(acc, B.part + (size_t)t * BATCH_PARTS);
    }
    if (!last_block(B.counter)) return;
    for (int s = threadIdx.x; s < B.S; s += BT) {
        KState *st = B.st + s;
        if (!st->active) continue;
        double tot[2];
        inst_sum<2>(B, s, tot);
        st->rur0[0] = tot[0];
        st->rur0[1] = tot[1];
    }
    __syncthreads();
    if (threadIdx.x == 0) *B.counter = 0u;
}

// ---------------------------------------------------------------- SpMV per tile
// y = A x on the rows of active instances (G lanes a row, 4 real / 2 complex: the
// lane count the single-system SpMV takes for the voxel systems; the lanes' sums
// combined by a fixed butterfly); with DOT also alpha = rur0 / (x . y).
template <typename T, bool DOT>
__global__ void __launch_bounds__(BT) k_bspmv(BDev B, const int *__restrict__ rp, const int *__restrict__ ci,
                                              const T *__restrict__ val, const T *__restrict__ x, T *__restrict__ y) {
    if (!B.ctl->active) return;
    constexpr int G = Sc<T>::is_complex ? 2 : 4, RPB = BT / G;
    const int g = threadIdx.x / G, gl = threadIdx.x % G;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        if (!B.act[(size_t)B.tile_sys[t] * B.act_stride]) continue;
        const int2 tr = B.tile[t];
        double acc2[2] = {0.0, 0.0};
        for (int row0 = tr.x; row0 < tr.y; row0 += RPB) {
            const int row = row0 + g;
            T acc = Sc<T>::zero();
            if (row < tr.y) {
                const int a = rp[row], e = rp[row + 1];
                for (int k = a + gl; k < e; k += G) acc = madd(acc, val[k], x[ci[k]]);
            }
#pragma unroll
            for (int m = G / 2; m >= 1; m >>= 1) acc = acc + Sc<T>::shfl_xor(acc, m);
            if (row < tr.y && gl == 0) {
                y[row] = acc;
                if (DOT) acc_parts<T>(acc2, x[row] * acc);
            }
        }
        if (DOT) block_partial<2>(acc2, B.part + (size_t)t * BATCH_PARTS);
    }
    if (!DOT || !last_block(B.counter)) return;
    for (int s = threadIdx.x; s < B.S; s += BT) {
        KState *st = B.st + s;
        if (!st->active) continue;
        double tot[2];
        inst_sum<2>(B, s, tot);
        st->dots[0] = tot[0];
        st->dots[1] = tot[1];
        using W = typename Wide<T>::type;
        putS<W>(st->alpha, getS<W>(st->rur0) / getS<W>(tot));
    }
    __syncthreads();
    if (threadIdx.x == 0) *B.counter = 0u;
}

// ---------------------------------------------------------------- ICCG steps
template <typename T>
__global__ void __launch_bounds__(BT) k_biccg_update(BDev B, T *x, T *r, const T *p, const T *ap) {
    if (!B.ctl->active) return;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        if (!B.act[(size_t)B.tile_sys[t] * B.act_stride]) continue;
        const KState *st = B.st + B.tile_sys[t];
        const T alpha = getS<T>(st->alpha);
        const int2 tr = B.tile[t];
        double acc[1] = {0.0};
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) {
            x[i] = x[i] + alpha * p[i];
            const T ri = r[i] - alpha * ap[i];
            r[i] = ri;
            acc[0] += Sc<T>::abs2(ri);
        }
        block_partial<1>(acc, B.part + (size_t)t * BATCH_PARTS);
    }
    if (!last_block(B.counter)) return;
    for (int s = threadIdx.x; s < B.S; s += BT) {
        KState *st = B.st + s;
        if (!st->active) continue;
        double tot[1];
        inst_sum<1>(B, s, tot);
        decide(st, sqrt(tot[0]), inst_log(B, s));
    }
    finish(B);
}

template <typename T>
__global__ void __launch_bounds__(BT) k_biccg_beta(BDev B, const T *r, const T *z) {
    if (!B.ctl->active) return;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        if (!B.act[(size_t)B.tile_sys[t] * B.act_stride]) continue;
        const int2 tr = B.tile[t];
        double acc[2] = {0.0, 0.0};
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) acc_parts<T>(acc, r[i] * z[i]);
        block_partial<2>(acc, B.part + (size_t)t * BATCH_PARTS);
    }
    if (!last_block(B.counter)) return;
    for (int s = threadIdx.x; s < B.S; s += BT) {
        KState *st = B.st + s;
        if (!st->active) continue;
        double tot[2];
        inst_sum<2>(B, s, tot);
        using W = typename Wide<T>::type;
        const W rur1 = getS<W>(tot);
        putS<W>(st->beta, rur1 / getS<W>(st->rur0));
        putS<W>(st->rur0, rur1);
    }
    __syncthreads();
    if (threadIdx.x == 0) *B.counter = 0u;
}

template <typename T>
__global__ void __launch_bounds__(BT) k_biccg_p(BDev B, T *p, const T *z) {
    if (!B.ctl->active) return;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        if (!B.act[(size_t)B.tile_sys[t] * B.act_stride]) continue;
        const KState *st = B.st + B.tile_sys[t];
        const T beta = getS<T>(st->beta);
        const int2 tr = B.tile[t];
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) p[i] = p[i] * beta + z[i];
    }
}

// ---------------------------------------------------------------- persistent ICCG (small instances)
// One CTA per instance runs all of its ICCG iterations: SpMV with p.Ap and alpha, the
// x / r update and the convergence test, the forward and backward IC sweeps level by
// level (a CTA barrier between levels), beta and the p update. Every piece does the
// arithmetic of the launch-per-phase kernels above in the same order (tile partials
// as 256-thread block sums added in tile order; the SpMV's 4 / 2 lanes a row; the
// sync-free sweep's G lanes a row, negated sums, lane 0 starting from the forward
// right-hand side, the same butterfly), so an instance gives the same bits either way;
// what goes away are the launches, the grid-wide reductions and the sweep's polling.
// An instance's rows stay in L2 between phases. No CTA waits on another.
constexpr int PERSIST_MAX_TILES = 8;  // instances of at most 8 tiles (16,384 rows)

struct BPer {
    const int *rp, *ci;
    const void *aval;
    const int *fperm, *fprp, *fpci;  // forward triangle in level order
    const void *fval, *dinv;         // its values; 1 / L_ii by row
    const int *bperm, *bprp, *bpci;  // backward triangle in level order
    const void *bval, *D;            // its values; D by row
    const int *flev, *blev;          // [S + 1]: first level range of each instance
    const int2 *frng, *brng;         // level ranges (positions in the level order) of each instance
    void *x, *r, *p, *z, *y, *v;
    int iters;                       // iterations to run at most
};

// one level range of a sweep: rows at positions [a, b), G lanes a row (k_sweep's arithmetic)
template <typename T, int G, int MODE>
__device__ __forceinline__ void persist_level(int a, int b, const int *perm, const int *prp, const int *pci,
                                              const T *val, const T *rhs, const T *aux, const T *Dv, const T *dinv,
                                              T *out) {
    const int g = threadIdx.x / G, gl = threadIdx.x % G;
    const unsigned gm = group_mask(G);
    for (int t = a + g; t < b; t += BT / G) {
        const int r = perm[t];
        const int ra = prp[t], re = prp[t + 1];
        constexpr bool fwd = MODE == SW_FWD_DIV;
        const int ob = fwd ? ra : ra + 1;
        const int oe = fwd ? (re > ra ? re - 1 : ra) : re;
        T acc = (fwd && gl == 0) ? rhs[r] : Sc<T>::zero();
        for (int k = ob + gl; k < oe; k += G) acc = madd(acc, -val[k], out[pci[k]]);
#pragma unroll
        for (int m = G / 2; m >= 1; m >>= 1) acc = acc + gshfl_xor(acc, m, gm);
        if (gl == 0) out[r] = fwd ? acc * dinv[r] : madd(aux[r], Dv[r], acc);
    }
}

template <typename T, int G>
__global__ void __launch_bounds__(BT) k_bpersist_iccg(BDev B, BPer P) {
    const int s = blockIdx.x;
    KState *st = B.st + s;
    __shared__ double tp[PERSIST_MAX_TILES][2];
    __shared__ int s_go;
    if (threadIdx.x == 0) s_go = st->active;
    __syncthreads();
    if (!s_go) return;
    using W = typename Wide<T>::type;
    const int t0 = B.sys_tile[s], t1 = B.sys_tile[s + 1];
    const T *aval = (const T *)P.aval;
    T *x = (T *)P.x, *r = (T *)P.r, *p = (T *)P.p, *z = (T *)P.z, *y = (T *)P.y, *v = (T *)P.v;
    double *log = inst_log(B, s);
    constexpr int GS = Sc<T>::is_complex ? 2 : 4, RPB = BT / GS;
    const int gs = threadIdx.x / GS, gls = threadIdx.x % GS;
    for (int it = 0; it < P.iters; ++it) {
        // SpMV v = A p with p . v per tile (k_bspmv), alpha = rur0 / (p . Ap)
        for (int t = t0; t < t1; ++t) {
            const int2 tr = B.tile[t];
            double acc2[2] = {0.0, 0.0};
            for (int row0 = tr.x; row0 < tr.y; row0 += RPB) {
                const int row = row0 + gs;
                T acc = Sc<T>::zero();
                if (row < tr.y) {
                    const int a = P.rp[row], e = P.rp[row + 1];
                    for (int k = a + gls; k < e; k += GS) acc = madd(acc, aval[k], p[P.ci[k]]);
                }
#pragma unroll
                for (int m = GS / 2; m >= 1; m >>= 1) acc = acc + Sc<T>::shfl_xor(acc, m);
                if (row < tr.y && gls == 0) {
                    v[row] = acc;
                    acc_parts<T>(acc2, p[row] * acc);
                }
            }
            block_partial<2>(acc2, tp[t - t0]);
        }
        if (threadIdx.x == 0) {
            double tot[2] = {0.0, 0.0};
            for (int t = t0; t < t1; ++t) {
                tot[0] += tp[t - t0][0];
                tot[1] += tp[t - t0][1];
            }
            st->dots[0] = tot[0];
            st->dots[1] = tot[1];
            putS<W>(st->alpha, getS<W>(st->rur0) / getS<W>(tot));
        }
        __syncthreads();
        // x += alpha p, r -= alpha Ap, |r| (k_biccg_update), the convergence test
        {
            const T alpha = getS<T>(st->alpha);
            for (int t = t0; t < t1; ++t) {
                const int2 tr = B.tile[t];
                double acc[1] = {0.0};
                for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) {
                    x[i] = x[i] + alpha * p[i];
                    const T ri = r[i] - alpha * v[i];
                    r[i] = ri;
                    acc[0] += Sc<T>::abs2(ri);
                }
                block_partial<1>(acc, tp[t - t0]);
            }
        }
        if (threadIdx.x == 0) {
            double tot = 0.0;
            for (int t = t0; t < t1; ++t) tot += tp[t - t0][0];
            decide(st, sqrt(tot), log);
            s_go = st->active;
        }
        __syncthreads();
        if (!s_go) break;
        // z = (L D L^T)^{-1} r: forward then backward, level by level
        for (int q = P.flev[s]; q < P.flev[s + 1]; ++q) {
            const int2 rg = P.frng[q];
            persist_level<T, G, SW_FWD_DIV>(rg.x, rg.y, P.fperm, P.fprp, P.fpci, (const T *)P.fval, r, nullptr,
                                            nullptr, (const T *)P.dinv, y);
            __syncthreads();
        }
        for (int q = P.blev[s]; q < P.blev[s + 1]; ++q) {
            const int2 rg = P.brng[q];
            persist_level<T, G, SW_BWD_IC>(rg.x, rg.y, P.bperm, P.bprp, P.bpci, (const T *)P.bval, nullptr, y,
                                           (const T *)P.D, nullptr, z);
            __syncthreads();
        }
        // beta = (r . z) / rur0 (k_biccg_beta), p = p beta + z (k_biccg_p)
        for (int t = t0; t < t1; ++t) {
            const int2 tr = B.tile[t];
            double acc[2] = {0.0, 0.0};
            for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) acc_parts<T>(acc, r[i] * z[i]);
            block_partial<2>(acc, tp[t - t0]);
        }
        if (threadIdx.x == 0) {
            double tot[2] = {0.0, 0.0};
            for (int t = t0; t < t1; ++t) {
                tot[0] += tp[t - t0][0];
                tot[1] += tp[t - t0][1];
            }
            const W rur1 = getS<W>(tot);
            putS<W>(st->beta, rur1 / getS<W>(st->rur0));
            putS<W>(st->rur0, rur1);
        }
        __syncthreads();
        {
            const T beta = getS<T>(st->beta);
            for (int t = t0; t < t1; ++t) {
                const int2 tr = B.tile[t];
                for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) p[i] = p[i] * beta + z[i];
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- IC-MRTR steps
template <typename T>
__global__ void __launch_bounds__(BT) k_bmrtr_dots(BDev B, const T *a, const T *b, const T *c, const T *y) {
    if (!B.ctl->active) return;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        if (!B.act[(size_t)B.tile_sys[t] * B.act_stride]) continue;
        const int2 tr = B.tile[t];
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) {
            const T ai = a[i];
            acc_parts<T>(acc + 0, ai * b[i]);
            acc_parts<T>(acc + 2, c[i] * ai);
            acc_parts<T>(acc + 4, ai * y[i]);
        }
        block_partial<6>(acc, B.part + (size_t)t * BATCH_PARTS);
    }
    if (!last_block(B.counter)) return;
    for (int s = threadIdx.x; s < B.S; s += BT) {
        KState *st = B.st + s;
        if (!st->active) continue;
        double tot[6];
        inst_sum<6>(B, s, tot);
        using W = typename Wide<T>::type;
        const W wr = getS<W>(tot + 0), vw = getS<W>(tot + 2), wy = getS<W>(tot + 4);
        for (int k = 0; k < 6; ++k) st->dots[k] = tot[k];
        W zeta, eta, nu = getS<W>(st->nu), zeta_old = getS<W>(st->zeta_old);
        if (st->it == 0) {
            zeta = wr / vw;
            zeta_old = zeta;
            eta = Sc<W>::zero();
        } else {
            const W temp0 = Sc<W>::one() / (nu * vw - wy * wy);
            zeta = nu * wr * temp0;
            eta = (-1.0 * wy) * wr * temp0;
        }
        nu = zeta * wr;
        const W ptemp = eta * zeta_old / zeta;
        zeta_old = zeta;
        putS<W>(st->zeta, zeta);
        putS<W>(st->eta, eta);
        putS<W>(st->nu, nu);
        putS<W>(st->ptemp, ptemp);
        putS<W>(st->zeta_old, zeta_old);
    }
    __syncthreads();
    if (threadIdx.x == 0) *B.counter = 0u;
}

template <typename T>
__global__ void __launch_bounds__(BT) k_bmrtr_update(BDev B, T *p, const T *u, T *x, T *y, const T *v, T *r) {
    if (!B.ctl->active) return;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        if (!B.act[(size_t)B.tile_sys[t] * B.act_stride]) continue;
        const KState *st = B.st + B.tile_sys[t];
        const T zeta = getS<T>(st->zeta), eta = getS<T>(st->eta), pt = getS<T>(st->ptemp);
        const int2 tr = B.tile[t];
        double acc[1] = {0.0};
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) {
            const T pi = p[i] * pt + u[i];
            p[i] = pi;
            x[i] = x[i] + zeta * pi;
            const T yi = y[i] * eta + zeta * v[i];
            y[i] = yi;
            const T ri = r[i] - yi;
            r[i] = ri;
            acc[0] += Sc<T>::abs2(ri);
        }
        block_partial<1>(acc, B.part + (size_t)t * BATCH_PARTS);
    }
    if (!last_block(B.counter)) return;
    for (int s = threadIdx.x; s < B.S; s += BT) {
        KState *st = B.st + s;
        if (!st->active) continue;
        double tot[1];
        inst_sum<1>(B, s, tot);
        decide(st, sqrt(tot[0]), inst_log(B, s));
    }
    finish(B);
}

template <typename T>
__global__ void __launch_bounds__(BT) k_bmrtr_zu(BDev B, T *z, const T *w, T *u) {
    if (!B.ctl->active) return;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        if (!B.act[(size_t)B.tile_sys[t] * B.act_stride]) continue;
        const KState *st = B.st + B.tile_sys[t];
        const T zeta = getS<T>(st->zeta), eta = getS<T>(st->eta);
        const int2 tr = B.tile[t];
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) {
            const T zi = z[i] * eta + zeta * w[i];
            z[i] = zi;
            u[i] = u[i] - zi;
        }
    }
}

// ---------------------------------------------------------------- mixed precision
// FP64 refinement around FP32 inner solves: per instance, r = b - A x in FP64,
// the inner solver (ICCG or IC-MRTR on FP32 copies of A and of the IC factor,
// FP32 vectors, FP64 scalars) reduces the scaled residual r / |r| by the inner
// tolerance, and x += |r| d in FP64, until |b - A x| / |b| reaches the
// tolerance. The factor and its shift are computed in FP64 and then rounded.
constexpr int MAX_OUTER = 40;

template <typename T, typename Ti>
__global__ void k_narrow(size_t n, const T *src, Ti *dst) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = to_lo(src[i]);
}

__device__ __forceinline__ void inner_reset(KState *st, double eta, int inner_max) {
    st->active = inner_max > 0 ? 1 : 0;
    st->status = inner_max > 0 ? ST_RUNNING : ST_MAXIT;
    st->it = 0;
    st->conv_cri = eta;
    st->normalizer = 1.0;  // the inner right-hand side is scaled to unit norm
    st->abs_conv_cri = 0.0;
    st->max_ite = inner_max;
    st->log_enabled = 0;
    st->best = 1.0e+6;
    st->bad_counter = 0;
    st->improved = 0;
    st->zeta[0] = st->zeta_old[0] = st->nu[0] = 1.0;
    st->zeta[1] = st->zeta_old[1] = st->nu[1] = 0.0;
    st->rur0[0] = st->rur0[1] = 0.0;
    // FP32 cannot take every inner solve to eta (the rounding of A and of the factor bounds
    // what one solve can gain); a stalled inner solve ends and the refinement continues
    st->stall_limit = 30;
    st->stall = 0;
    st->stall_best = 1.0e+300;
}

// after k_bsetup (one block): refinement state of every instance, first inner solve armed
__global__ void k_bmix_begin(BDev B, OState *O, KState *octl, double eta, int inner_max) {
    int any = 0;
    for (int s = threadIdx.x; s < B.S; s += blockDim.x) {
        KState *st = B.st + s;
        OState *o = O + s;
        o->active = st->active;
        o->status = st->status;
        o->outer_it = 0;
        o->inner_total = 0;
        o->normB = o->norm = o->scale = st->normalizer;
        if (st->active) {
            inner_reset(st, eta, inner_max);
            any = 1;
        }
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) {
        octl->active = any;
        B.ctl->active = any;
    }
}

// inner right-hand side r / |r| in FP32 and a zero inner solution (outer-active instances)
template <typename T, typename Ti>
__global__ void __launch_bounds__(BT) k_bscale(BDev Bo, const OState *O, const T *r, Ti *rin, Ti *d) {
    if (!Bo.ctl->active) return;
    for (int t = blockIdx.x; t < Bo.NT; t += gridDim.x) {
        const int s = Bo.tile_sys[t];
        if (!Bo.act[(size_t)s * Bo.act_stride]) continue;
        const double inv = 1.0 / O[s].scale;
        const int2 tr = Bo.tile[t];
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) {
            rin[i] = to_lo(inv * r[i]);
            d[i] = Sc<Ti>::zero();
        }
    }
}

// x += |r| d in FP64
template <typename T, typename Ti>
__global__ void __launch_bounds__(BT) k_bouter_update(BDev Bo, const OState *O, T *x, const Ti *d) {
    if (!Bo.ctl->active) return;
    for (int t = blockIdx.x; t < Bo.NT; t += gridDim.x) {
        const int s = Bo.tile_sys[t];
        if (!Bo.act[(size_t)s * Bo.act_stride]) continue;
        const double sc = O[s].scale;
        const int2 tr = Bo.tile[t];
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) x[i] = x[i] + sc * to_hi(d[i]);
    }
}

// r = b - A x (v = A x), |r| per instance, the refinement decision; a continuing
// instance gets its next inner solve armed
template <typename T>
__global__ void __launch_bounds__(BT) k_bresid(BDev Bo, OState *O, KState *ictl, const T *b, const T *v, T *r,
                                               double tol, int max_ite, double eta) {
    if (!Bo.ctl->active) return;
    for (int t = blockIdx.x; t < Bo.NT; t += gridDim.x) {
        if (!Bo.act[(size_t)Bo.tile_sys[t] * Bo.act_stride]) continue;
        const int2 tr = Bo.tile[t];
        double acc[1] = {0.0};
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) {
            const T ri = b[i] - v[i];
            r[i] = ri;
            acc[0] += Sc<T>::abs2(ri);
        }
        block_partial<1>(acc, Bo.part + (size_t)t * BATCH_PARTS);
    }
    if (!last_block(Bo.counter)) return;
    int any = 0;
    for (int s = threadIdx.x; s < Bo.S; s += BT) {
        OState *o = O + s;
        if (!o->active) continue;
        KState *st = Bo.st + s;
        double tot[1];
        inst_sum<1>(Bo, s, tot);
        const double norm = sqrt(tot[0]);
        o->outer_it += 1;
        o->inner_total += st->it;
        inst_log(Bo, s)[o->outer_it] = norm / o->normB;
        if (norm / o->normB < tol) {
            o->active = 0;
            o->status = ST_CONVERGED;
        } else if (o->inner_total >= max_ite || o->outer_it >= MAX_OUTER) {
            o->active = 0;
            o->status = ST_MAXIT;
        } else {
            o->norm = o->scale = norm;
            inner_reset(st, eta, max_ite - o->inner_total);
            any = 1;
        }
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) {
        Bo.ctl->active = any;
        ictl->active = any;
        *Bo.counter = 0u;
    }
}

template <typename T>
__global__ void __launch_bounds__(BT) k_bneg(BDev B, const T *a, T *out) {
    if (!B.ctl->active) return;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        if (!B.act[(size_t)B.tile_sys[t] * B.act_stride]) continue;
        const int2 tr = B.tile[t];
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) out[i] = Sc<T>::zero() - a[i];
    }
}

// ---------------------------------------------------------------- host side
static int bgrid(int NT) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return std::max(1, std::min(NT, sms * 8));
}

Batch::Batch(int dev) : h(dev) {
    // fixed lanes per row in both sweep schedules and in the SpMV: an
    // instance's arithmetic must not depend on the batch it is in
    h.swcfg.group = 8;
    h.cl_group = 8;
    h.push_auto = false;
    SSG_CUDA(cudaEventCreateWithFlags(&ev_chunk, cudaEventDisableTiming));
    for (auto &e : ev) SSG_CUDA(cudaEventCreate(&e));
    SSG_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
}

void Batch::drop_graph() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
}

Batch::~Batch() {
    cudaSetDevice(h.device);
    drop_graph();
    if (h_st) cudaFreeHost(h_st);
    if (h_ctl) cudaFreeHost(h_ctl);
    if (h_octl) cudaFreeHost(h_octl);
    if (h_ost) cudaFreeHost(h_ost);
    if (ev_chunk) cudaEventDestroy(ev_chunk);
    if (side) cudaStreamDestroy(side);
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
}

int Batch::add(int n, int nnz, const int *rp, const int *ci, const double *val, int vt, int nrhs, const double *B) {
    if (running) throw Error{SSG_ERR_STATE, "batch is running"};
    if (n <= 0 || nnz < n || nrhs < 1 || !rp || !ci || !val || !B) throw Error{SSG_ERR_ARG, "bad system arguments"};
    if (vt != SSG_REAL && vt != SSG_COMPLEX) throw Error{SSG_ERR_ARG, "bad value type"};
    if (vtype >= 0 && vt != vtype) throw Error{SSG_ERR_ARG, "a batch holds only real or only complex systems"};
    if (rp[0] != 0 || rp[n] != nnz) throw Error{SSG_ERR_ARG, "row pointers do not span the entries"};
    const int w = vt == SSG_COMPLEX ? 2 : 1;
    BatchSystem S_;
    S_.n = n;
    S_.nnz = nnz;
    S_.nrhs = nrhs;
    S_.rp.assign(rp, rp + n + 1);
    S_.ci.assign(ci, ci + nnz);
    S_.val.assign(val, val + (size_t)w * nnz);
    S_.B.assign(B, B + (size_t)w * n * nrhs);
    sys.push_back(std::move(S_));
    vtype = vt;
    assembled = false;
    rhs_dirty = true;
    return (int)sys.size() - 1;
}

void Batch::set_rhs(int index, const double *B) {
    if (running) throw Error{SSG_ERR_STATE, "batch is running"};
    if (index < 0 || index >= (int)sys.size() || !B) throw Error{SSG_ERR_ARG, "bad system index"};
    BatchSystem &q = sys[index];
    std::memcpy(q.B.data(), B, sizeof(double) * q.B.size());
    rhs_dirty = true;
}

void Batch::set_rhs_device(int index, const void *dB) {
    if (running) throw Error{SSG_ERR_STATE, "batch is running"};
    if (index < 0 || index >= (int)sys.size() || !dB) throw Error{SSG_ERR_ARG, "bad system index"};
    dev_rhs.resize(sys.size(), nullptr);
    dev_rhs[index] = dB;
}

void Batch::result_device(int index, void *dX) {
    if (running) throw Error{SSG_ERR_STATE, "batch is running"};
    if (index < 0 || index >= (int)sys.size() || !dX) throw Error{SSG_ERR_ARG, "bad system index"};
    const size_t vb = vtype == SSG_COMPLEX ? 16 : 8;
    for (int q = 0; q < S; ++q) {
        if (inst_sys[q] != index) continue;
        const int n = sys[index].n;
        SSG_CUDA(cudaMemcpyAsync((char *)dX + vb * (size_t)n * inst_rhs[q], h.vec[8].as<char>() + vb * (size_t)inst_row[q],
                                 vb * (size_t)n, cudaMemcpyDeviceToDevice, h.stream));
    }
    SSG_CUDA(cudaStreamSynchronize(h.stream));
}

void Batch::update_values_device(int index, const void *dval) {
    if (running) throw Error{SSG_ERR_STATE, "batch is running"};
    if (index < 0 || index >= (int)sys.size() || !dval) throw Error{SSG_ERR_ARG, "bad system index"};
    if (!assembled) throw Error{SSG_ERR_STATE, "batch not assembled"};
    const size_t vb = vtype == SSG_COMPLEX ? 16 : 8;
    for (int q = 0; q < S; ++q) {
        if (inst_sys[q] != index) continue;
        SSG_CUDA(cudaMemcpyAsync(h.A_val.as<char>() + vb * (size_t)inst_entry[q], dval, vb * (size_t)sys[index].nnz,
                                 cudaMemcpyDeviceToDevice, h.stream));
    }
    SSG_CUDA(cudaStreamSynchronize(h.stream));
    h.values_changed();
}

void Batch::clear() {
    if (running) throw Error{SSG_ERR_STATE, "batch is running"};
    sys.clear();
    vtype = -1;
    assembled = false;
}

// block-diagonal matrix of all instances, tiles, per-instance buffers
void Batch::assemble() {
    if (sys.empty()) throw Error{SSG_ERR_STATE, "empty batch"};
    const int w = vtype == SSG_COMPLEX ? 2 : 1;
    inst_sys.clear();
    inst_rhs.clear();
    inst_row.assign(1, 0);
    inst_entry.clear();
    long long N = 0, NNZ = 0;
    for (size_t q = 0; q < sys.size(); ++q)
        for (int j = 0; j < sys[q].nrhs; ++j) {
            inst_sys.push_back((int)q);
            inst_rhs.push_back(j);
            inst_entry.push_back(NNZ);
            N += sys[q].n;
            NNZ += sys[q].nnz;
            if (N >= (1ll << 31) - 1 || NNZ >= (1ll << 31) - 1)
                throw Error{SSG_ERR_ARG, "batch exceeds 2^31 rows or entries"};
            inst_row.push_back((int)N);
        }
    S = (int)inst_sys.size();
    std::vector<int> rp((size_t)N + 1), ci((size_t)NNZ);
    std::vector<double> val((size_t)w * NNZ);
    std::vector<int2> tiles;
    std::vector<int> tile_sys, sys_tile(1, 0);
    long long e = 0;
    for (int s = 0; s < S; ++s) {
        const BatchSystem &q = sys[inst_sys[s]];
        const int r0 = inst_row[s];
        for (int i = 0; i < q.n; ++i) rp[(size_t)r0 + i] = (int)(e + q.rp[i]);
        for (int k = 0; k < q.nnz; ++k) ci[(size_t)e + k] = q.ci[k] + r0;
        std::memcpy(val.data() + (size_t)w * e, q.val.data(), sizeof(double) * (size_t)w * q.nnz);
        e += q.nnz;
        for (int t0 = 0; t0 < q.n; t0 += BATCH_TILE) {
            tiles.push_back(make_int2(r0 + t0, r0 + std::min(q.n, t0 + BATCH_TILE)));
            tile_sys.push_back(s);
        }
        sys_tile.push_back((int)tiles.size());
    }
    rp[(size_t)N] = (int)e;
    NT = (int)tiles.size();
    h_sys_tile = sys_tile;
    pr_key = ~0ull;
    h.set_matrix((int)N, (int)NNZ, rp.data(), ci.data(), val.data(), vtype, cudaMemcpyHostToDevice);
    // a system's instances for its second and later right-hand sides have the same matrix
    // as its first: their factor rows are copies of the first instance's
    std::vector<int> rep;
    for (int s = 0; s < S; ++s) {
        if (inst_rhs[s] == 0) continue;
        if (rep.empty()) rep.assign((size_t)N, -1);
        const int src0 = inst_row[s - inst_rhs[s]];
        for (int i = 0; i < sys[inst_sys[s]].n; ++i) rep[(size_t)inst_row[s] + i] = src0 + i;
    }
    h.set_replicas(rep);
    d_tile.ensure(sizeof(int2) * (size_t)NT);
    d_tile_sys.ensure(sizeof(int) * (size_t)NT);
    d_sys_tile.ensure(sizeof(int) * (size_t)(S + 1));
    d_sys_row.ensure(sizeof(int) * (size_t)(S + 1));
    d_st.ensure(sizeof(KState) * (size_t)S);
    d_part.ensure(sizeof(double) * BATCH_PARTS * (size_t)NT);
    d_ctl_counter.ensure(sizeof(KState) + 64);
    cudaStream_t st = h.stream;
    SSG_CUDA(cudaMemcpyAsync(d_tile.p, tiles.data(), sizeof(int2) * (size_t)NT, cudaMemcpyHostToDevice, st));
    SSG_CUDA(cudaMemcpyAsync(d_tile_sys.p, tile_sys.data(), sizeof(int) * (size_t)NT, cudaMemcpyHostToDevice, st));
    SSG_CUDA(cudaMemcpyAsync(d_sys_tile.p, sys_tile.data(), sizeof(int) * (size_t)(S + 1), cudaMemcpyHostToDevice, st));
    SSG_CUDA(cudaMemcpyAsync(d_sys_row.p, inst_row.data(), sizeof(int) * (size_t)(S + 1), cudaMemcpyHostToDevice, st));
    SSG_CUDA(cudaMemsetAsync(d_ctl_counter.p, 0, sizeof(KState) + 64, st));
    {
        std::vector<int> row_inst((size_t)N);
        for (int q = 0; q < S; ++q)
            std::fill(row_inst.begin() + inst_row[q], row_inst.begin() + inst_row[q + 1], q);
        d_row_inst.ensure(sizeof(int) * ((size_t)N + 1));
        SSG_CUDA(cudaMemcpyAsync(d_row_inst.p, row_inst.data(), sizeof(int) * (size_t)N, cudaMemcpyHostToDevice, st));
        SSG_CUDA(cudaStreamSynchronize(st));  // row_inst is freed at the end of this scope
        h.swcfg.row_inst = d_row_inst.as<int>();
        h.swcfg.act = &d_st.as<KState>()->active;
        h.swcfg.act_stride = (int)(sizeof(KState) / sizeof(int));
    }
    // pinned copies grow only: freeing pinned memory waits for the whole device
    if (S > h_cap) {
        if (h_st) cudaFreeHost(h_st);
        if (h_ost) cudaFreeHost(h_ost);
        h_st = nullptr;
        h_ost = nullptr;
        const int cap = std::max(S, 2 * h_cap);
        SSG_CUDA(cudaMallocHost((void **)&h_st, sizeof(KState) * (size_t)cap));
        SSG_CUDA(cudaMallocHost((void **)&h_ost, sizeof(OState) * (size_t)cap));
        h_cap = cap;
    }
    if (!h_ctl) SSG_CUDA(cudaMallocHost((void **)&h_ctl, sizeof(KState)));
    if (!h_octl) SSG_CUDA(cudaMallocHost((void **)&h_octl, sizeof(KState)));
    d_ost.ensure(sizeof(OState) * (size_t)S);
    d_octl.ensure(sizeof(KState));
    SSG_CUDA(cudaStreamSynchronize(st));
    assembled = true;
}

KState *Batch::ctl() { return d_ctl_counter.as<KState>(); }

BDev Batch::dev_view() {
    BDev B;
    B.S = S;
    B.NT = NT;
    B.tile = d_tile.as<int2>();
    B.tile_sys = d_tile_sys.as<int>();
    B.sys_tile = d_sys_tile.as<int>();
    B.sys_row = d_sys_row.as<int>();
    B.st = d_st.as<KState>();
    B.act = &d_st.as<KState>()->active;
    B.act_stride = (int)(sizeof(KState) / sizeof(int));
    B.ctl = ctl();
    B.part = d_part.as<double>();
    B.counter = (unsigned *)(d_ctl_counter.as<char>() + sizeof(KState));
    B.logs = d_logs.as<double>();
    B.log_stride = max_ite + 2 + MAX_OUTER;
    return B;
}

template <typename T>
void Batch::start(int method_, double alpha, double conv, int max_ite_) {
    if (running) throw Error{SSG_ERR_STATE, "batch is running"};
    if (method_ != SSG_METHOD_ICCG && method_ != SSG_METHOD_MRTR) throw Error{SSG_ERR_ARG, "bad method"};
    if (!(alpha > 0.0)) throw Error{SSG_ERR_ARG, "a batch needs a fixed shift alpha > 0"};
    if (max_ite_ < 0 || !(conv > 0.0)) throw Error{SSG_ERR_ARG, "bad tolerance or iteration limit"};
    if (!assembled) assemble();
    method = method_;
    max_ite = max_ite_;
    cudaStream_t s = h.stream;
    drop_graph();  // buffers and plans may have changed since the last start
    SSG_CUDA(cudaEventRecord(ev[0], s));
    const int n = h.n;
    // the factor is recomputed on every start, as the reference's solve() does
    h.fac_valid = false;
    h.ensure_factor<T>(alpha, false);
    h.ensure_work(sizeof(T));
    d_logs.ensure(sizeof(double) * (size_t)S * (size_t)(max_ite + 2 + MAX_OUTER));
    T *b = h.vec[0].as<T>(), *r = h.vec[1].as<T>(), *p = h.vec[2].as<T>(), *z = h.vec[3].as<T>();
    T *u = h.vec[4].as<T>(), *y = h.vec[5].as<T>(), *x = h.vec[8].as<T>();
    // right-hand sides of all instances, uploaded when they changed (they stay resident otherwise)
    if (rhs_dirty) {
        const int w = vtype == SSG_COMPLEX ? 2 : 1;
        std::vector<double> stage((size_t)w * n);
        for (int q = 0; q < S; ++q) {
            const BatchSystem &sy = sys[inst_sys[q]];
            std::memcpy(stage.data() + (size_t)w * inst_row[q], sy.B.data() + (size_t)w * sy.n * inst_rhs[q],
                        sizeof(double) * (size_t)w * sy.n);
        }
        SSG_CUDA(cudaMemcpyAsync(b, stage.data(), sizeof(T) * (size_t)n, cudaMemcpyHostToDevice, s));
        SSG_CUDA(cudaStreamSynchronize(s));
        rhs_dirty = false;
    }
    // right-hand sides given in device memory
    for (size_t i = 0; i < dev_rhs.size(); ++i) {
        if (!dev_rhs[i]) continue;
        for (int q = 0; q < S; ++q) {
            if (inst_sys[q] != (int)i) continue;
            const int ns = sys[i].n;
            SSG_CUDA(cudaMemcpyAsync(b + inst_row[q], (const T *)dev_rhs[i] + (size_t)ns * inst_rhs[q],
                                     sizeof(T) * (size_t)ns, cudaMemcpyDeviceToDevice, s));
        }
        dev_rhs[i] = nullptr;
    }
    for (int q = 0; q < S; ++q) {
        KState &k = h_st[q];
        std::memset(&k, 0, sizeof(KState));
        k.active = 1;
        k.status = ST_RUNNING;
        k.max_ite = max_ite;
        k.bad_div_count_thres = 1000;
        k.bad_div_val = 1000.0;
        k.log_enabled = 1;
        k.conv_cri = conv;
        k.best = 1.0e+6;
        k.zeta[0] = k.zeta_old[0] = k.nu[0] = 1.0;
        k.log_len = -1;
    }
    std::memset(h_ctl, 0, sizeof(KState));
    h_ctl->active = 1;
    seen_st.clear();
    seen_ost.clear();
    SSG_CUDA(cudaMemcpyAsync(d_st.p, h_st, sizeof(KState) * (size_t)S, cudaMemcpyHostToDevice, s));
    SSG_CUDA(cudaMemcpyAsync(ctl(), h_ctl, sizeof(KState), cudaMemcpyHostToDevice, s));
    SSG_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * (size_t)n, s));
    SSG_CUDA(cudaMemcpyAsync(r, b, sizeof(T) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    BDev B = dev_view();
    const int grid = bgrid(NT);
    const double nv = (double)sizeof(T) * n;
    h.prof.iter = 0;
    h.prof.pre = true;
    iter_no = 0;
    h.timed(PC_VEC, nv, [&] {
        k_bsetup<T><<<grid, BT, 0, s>>>(B, b);
        SSG_LAUNCHED();
    });
    conv_cri = conv;
    if (precision == SSG_PREC_MIXED) {
        using Ti = typename Lo<T>::type;
        start_mixed<T, Ti>(alpha, conv);
        SSG_CUDA(cudaEventRecord(ev[1], s));
        queued = 0;
        chunk = 2;
        running = true;
        queue_inner<T, Ti>(chunk);
        return;
    }
    if (method == SSG_METHOD_ICCG) {
        h.apply_precond<T>(r, z, ctl());
        SSG_CUDA(cudaMemcpyAsync(p, z, sizeof(T) * (size_t)n, cudaMemcpyDeviceToDevice, s));
        h.timed(PC_VEC, 2 * nv, [&] {
            k_brur0<T><<<grid, BT, 0, s>>>(B, r, z);
            SSG_LAUNCHED();
        });
    } else {
        h.apply_precond<T>(r, u, ctl());
        vec_neg<T>(n, r, y, s);
        h.apply_precond<T>(y, z, ctl());
        SSG_CUDA(cudaMemsetAsync(p, 0, sizeof(T) * (size_t)n, s));
    }
    SSG_CUDA(cudaEventRecord(ev[1], s));
    queued = 0;
    chunk = 2;
    running = true;
    queue_chunk<T>();
}

bool Batch::persist_ok() const {
    if (!persist || method != SSG_METHOD_ICCG || precision != SSG_PREC_FP64 || h.prof.on || !h.use_inv_diag) return false;
    const int G = h.swcfg.group;
    if (G != 4 && G != 8 && G != 16 && G != 32) return false;
    if ((int)h_sys_tile.size() != S + 1) return false;
    for (int q = 0; q < S; ++q)
        if (h_sys_tile[q + 1] - h_sys_tile[q] > PERSIST_MAX_TILES) return false;
    return true;
}

// each instance's rows of each level of the forward and backward triangles: within a
// level the rows are in row order and an instance's rows are contiguous, so each
// (level, instance) is one range of positions; an instance's ranges in level order
void Batch::persist_ranges() {
    if (pr_key == h.pattern_id) return;
    const int n = h.n;
    std::vector<int> rinst((size_t)n);
    for (int q = 0; q < S; ++q)
        for (int i = inst_row[q]; i < inst_row[q + 1]; ++i) rinst[i] = q;
    auto build = [&](const Tri &T, DBuf &dl, DBuf &dr) {
        std::vector<int> perm((size_t)n);
        if (n) SSG_CUDA(cudaMemcpy(perm.data(), T.perm.p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost));
        std::vector<int> first((size_t)S + 1, 0);
        std::vector<int3> runs;  // (instance, start, end)
        for (int L = 0; L < T.nlev; ++L)
            for (int t = T.lptr[L]; t < T.lptr[L + 1];) {
                const int q = rinst[perm[t]];
                int e = t + 1;
                while (e < T.lptr[L + 1] && rinst[perm[e]] == q) ++e;
                runs.push_back(make_int3(q, t, e));
                ++first[q + 1];
                t = e;
            }
        for (int q = 0; q < S; ++q) first[q + 1] += first[q];
        std::vector<int2> rng(runs.size() + 1, make_int2(0, 0));
        std::vector<int> fill(first.begin(), first.end() - 1);
        for (const int3 &r : runs) rng[fill[r.x]++] = make_int2(r.y, r.z);
        dl.ensure(sizeof(int) * (first.size()));
        dr.ensure(sizeof(int2) * rng.size());
        SSG_CUDA(cudaMemcpy(dl.p, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice));
        SSG_CUDA(cudaMemcpy(dr.p, rng.data(), sizeof(int2) * rng.size(), cudaMemcpyHostToDevice));
    };
    build(h.Lf, d_pl_f, d_pr_f);
    build(h.Ltb, d_pl_b, d_pr_b);
    pr_key = h.pattern_id;
}

template <typename T>
void Batch::queue_persistent() {
    cudaStream_t s = h.stream;
    persist_ranges();
    BDev B = dev_view();
    BPer P;
    P.rp = h.A_rp.as<int>();
    P.ci = h.A_ci.as<int>();
    P.aval = h.A_val.p;
    P.fperm = h.Lf.perm.as<int>();
    P.fprp = h.Lf.prp.as<int>();
    P.fpci = h.Lf.pci.as<int>();
    P.fval = h.Lval.p;
    P.dinv = h.invL.p;
    P.bperm = h.Ltb.perm.as<int>();
    P.bprp = h.Ltb.prp.as<int>();
    P.bpci = h.Ltb.pci.as<int>();
    P.bval = h.Ltval.p;
    P.D = h.Dvec.p;
    P.flev = d_pl_f.as<int>();
    P.frng = d_pr_f.as<int2>();
    P.blev = d_pl_b.as<int>();
    P.brng = d_pr_b.as<int2>();
    P.x = h.vec[8].p;
    P.r = h.vec[1].p;
    P.p = h.vec[2].p;
    P.z = h.vec[3].p;
    P.y = h.vec[10].p;
    P.v = h.vec[6].p;
    P.iters = max_ite - queued;
    if (S > 0 && P.iters > 0) {
        switch (h.swcfg.group) {
            case 4: k_bpersist_iccg<T, 4><<<S, BT, 0, s>>>(B, P); break;
            case 8: k_bpersist_iccg<T, 8><<<S, BT, 0, s>>>(B, P); break;
            case 16: k_bpersist_iccg<T, 16><<<S, BT, 0, s>>>(B, P); break;
            default: k_bpersist_iccg<T, 32><<<S, BT, 0, s>>>(B, P); break;
        }
        SSG_LAUNCHED();
    }
    queued = max_ite;
    SSG_CUDA(cudaMemcpyAsync(h_ctl, ctl(), sizeof(KState), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaMemcpyAsync(h_st, d_st.p, sizeof(KState) * (size_t)S, cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaEventRecord(ev_chunk, s));
}

template <typename T>
void Batch::queue_chunk() {
    if (persist_ok()) {
        queue_persistent<T>();
        return;
    }
    cudaStream_t s = h.stream;
    const int n = h.n;
    BDev B = dev_view();
    const int grid = bgrid(NT);
    const int *rp = h.A_rp.as<int>(), *ci = h.A_ci.as<int>();
    const T *aval = h.A_val.as<T>();
    T *r = h.vec[1].as<T>(), *p = h.vec[2].as<T>(), *z = h.vec[3].as<T>(), *u = h.vec[4].as<T>();
    T *y = h.vec[5].as<T>(), *v = h.vec[6].as<T>(), *w = h.vec[7].as<T>(), *x = h.vec[8].as<T>();
    const int todo = std::min(chunk, max_ite - queued);
    const double nv = (double)sizeof(T) * n;
    const double spmv_bytes = (4.0 + sizeof(T)) * h.nnz + 4.0 * (n + 1) + 2.0 * nv;
    run_iterations(todo, [&] {
        h.prof.iter = ++iter_no;
        h.prof.pre = true;
        if (method == SSG_METHOD_ICCG) {
            h.timed(PC_SPMV, spmv_bytes, [&] {
                k_bspmv<T, true><<<grid, BT, 0, s>>>(B, rp, ci, aval, p, v);
                SSG_LAUNCHED();
            });
            h.timed(PC_VEC, 6 * nv, [&] {
                k_biccg_update<T><<<grid, BT, 0, s>>>(B, x, r, p, v);
                SSG_LAUNCHED();
            });
            h.prof.pre = false;
            h.apply_precond<T>(r, z, ctl());
            h.timed(PC_VEC, 2 * nv, [&] {
                k_biccg_beta<T><<<grid, BT, 0, s>>>(B, r, z);
                SSG_LAUNCHED();
            });
            h.timed(PC_VEC, 3 * nv, [&] {
                k_biccg_p<T><<<grid, BT, 0, s>>>(B, p, z);
                SSG_LAUNCHED();
            });
        } else {
            h.timed(PC_SPMV, spmv_bytes, [&] {
                k_bspmv<T, false><<<grid, BT, 0, s>>>(B, rp, ci, aval, u, v);
                SSG_LAUNCHED();
            });
            h.apply_precond<T>(v, w, ctl());
            h.timed(PC_VEC, 4 * nv, [&] {
                k_bmrtr_dots<T><<<grid, BT, 0, s>>>(B, w, r, v, y);
                SSG_LAUNCHED();
            });
            h.timed(PC_VEC, 10 * nv, [&] {
                k_bmrtr_update<T><<<grid, BT, 0, s>>>(B, p, u, x, y, v, r);
                SSG_LAUNCHED();
            });
            h.prof.pre = false;
            h.timed(PC_VEC, 5 * nv, [&] {
                k_bmrtr_zu<T><<<grid, BT, 0, s>>>(B, z, w, u);
                SSG_LAUNCHED();
            });
        }
    });
    queued += todo;
    chunk = std::min(chunk * 2, 32);
    SSG_CUDA(cudaMemcpyAsync(h_ctl, ctl(), sizeof(KState), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaMemcpyAsync(h_st, d_st.p, sizeof(KState) * (size_t)S, cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaEventRecord(ev_chunk, s));
}

bool Batch::poll() {
    if (!running) return true;
    const cudaError_t q = cudaEventQuery(ev_chunk);
    if (q == cudaErrorNotReady) return false;
    SSG_CUDA(q);
    h.check_err("batched iterations");
    seen_st.assign(h_st, h_st + S);
    if (precision == SSG_PREC_MIXED) seen_ost.assign(h_ost, h_ost + S);
    if (precision == SSG_PREC_MIXED) {
        const bool cx = vtype == SSG_COMPLEX;
        if (h_ctl->active && queued < max_ite) {
            if (cx)
                queue_inner<cplx, cplxf>(chunk);
            else
                queue_inner<double, float>(chunk);
            return false;
        }
        if (h_octl->active) {
            queued = 0;
            chunk = 2;
            if (cx) {
                queue_outer_step<cplx, cplxf>();
                queue_inner<cplx, cplxf>(chunk);
            } else {
                queue_outer_step<double, float>();
                queue_inner<double, float>(chunk);
            }
            return false;
        }
    } else if (h_ctl->active && queued < max_ite) {
        if (vtype == SSG_COMPLEX)
            queue_chunk<cplx>();
        else
            queue_chunk<double>();
        return false;
    }
    cudaStream_t s = h.stream;
    SSG_CUDA(cudaMemcpyAsync(h_st, d_st.p, sizeof(KState) * (size_t)S, cudaMemcpyDeviceToHost, s));
    if (precision == SSG_PREC_MIXED)
        SSG_CUDA(cudaMemcpyAsync(h_ost, d_ost.p, sizeof(OState) * (size_t)S, cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaEventRecord(ev[2], s));
    SSG_CUDA(cudaStreamSynchronize(s));
    int most = 0;
    for (int q = 0; q < S; ++q) most = std::max(most, h_st[q].it);
    if (precision == SSG_PREC_MIXED) most = 1 << 30;  // every profiled launch of a refinement did work
    seen_st.assign(h_st, h_st + S);
    if (precision == SSG_PREC_MIXED) seen_ost.assign(h_ost, h_ost + S);
    h.prof_flush(most);
    h.prof.iter = 0;
    float a = 0.f, b = 0.f;
    cudaEventElapsedTime(&a, ev[0], ev[1]);
    cudaEventElapsedTime(&b, ev[1], ev[2]);
    t_ms = {a, b};
    running = false;
    return true;
}

void Batch::wait() {
    while (!poll()) SSG_CUDA(cudaEventSynchronize(ev_chunk));
}

bool Batch::step() {
    if (!running) return true;
    SSG_CUDA(cudaEventSynchronize(ev_chunk));
    return poll();
}

bool Batch::finished(int index) const {
    if (index < 0 || index >= (int)sys.size()) throw Error{SSG_ERR_ARG, "bad system index"};
    if (!running) return !t_ms.empty();
    const bool mixed = precision == SSG_PREC_MIXED;
    if ((int)seen_st.size() != S || (mixed && (int)seen_ost.size() != S)) return false;
    for (int q = 0; q < S; ++q)
        if (inst_sys[q] == index && (mixed ? seen_ost[q].active : seen_st[q].active)) return false;
    return true;
}

// Allowed while the batch runs once the system's instances ended: their rows of
// x are no longer written (every update kernel skips ended instances).
int Batch::result(int index, double *X, int *iters, int *status) {
    if (index < 0 || index >= (int)sys.size()) throw Error{SSG_ERR_ARG, "bad system index"};
    if (!assembled || (!running && t_ms.empty())) throw Error{SSG_ERR_STATE, "no finished solve"};
    if (running && !finished(index)) throw Error{SSG_ERR_STATE, "system still running"};
    cudaStream_t cs = running ? side : h.stream;
    const size_t vb = vtype == SSG_COMPLEX ? 16 : 8;
    int rc = SSG_OK;
    for (int q = 0; q < S; ++q) {
        if (inst_sys[q] != index) continue;
        const int j = inst_rhs[q], n = sys[index].n;
        if (X)
            SSG_CUDA(cudaMemcpyAsync((char *)X + vb * (size_t)n * j, h.vec[8].as<char>() + vb * (size_t)inst_row[q],
                                     vb * (size_t)n, cudaMemcpyDeviceToHost, cs));
        const bool mixed = precision == SSG_PREC_MIXED;
        const int it = mixed ? seen_ost[q].inner_total : seen_st[q].it;
        const int stt = mixed ? seen_ost[q].status : seen_st[q].status;
        if (iters) iters[j] = it;
        if (status) status[j] = stt;
        if (stt != ST_CONVERGED) rc = SSG_NOT_CONVERGED;
    }
    SSG_CUDA(cudaStreamSynchronize(cs));
    return rc;
}

int Batch::instance(int index, int rhs) const {
    for (int q = 0; q < S; ++q)
        if (inst_sys[q] == index && inst_rhs[q] == rhs) return q;
    return -1;
}

int Batch::residual_log(int index, int rhs, double *out, int capacity, int *length) {
    if (running) throw Error{SSG_ERR_STATE, "batch is running"};
    if (!assembled || t_ms.empty()) throw Error{SSG_ERR_STATE, "no finished solve"};
    const int q = instance(index, rhs);
    if (q < 0) throw Error{SSG_ERR_ARG, "bad system index or right-hand side"};
    // mixed precision: the log holds |b - A x| / |b| after each refinement step
    const int len = seen_st[q].log_len >= 0 ? seen_st[q].log_len
                    : (precision == SSG_PREC_MIXED ? seen_ost[q].outer_it + 1 : seen_st[q].it + 1);
    if (length) *length = len;
    if (out && capacity > 0) {
        const int m = std::min(capacity, len);
        if (m > 0)
            SSG_CUDA(cudaMemcpy(out, d_logs.as<double>() + (size_t)q * (max_ite + 2 + MAX_OUTER), sizeof(double) * (size_t)m,
                                cudaMemcpyDeviceToHost));
    }
    return SSG_OK;
}

// ---------------------------------------------------------------- mixed precision, host side
BDev Batch::outer_view() {
    BDev B = dev_view();
    B.act = &d_ost.as<OState>()->active;
    B.act_stride = (int)(sizeof(OState) / sizeof(int));
    B.ctl = octl();
    return B;
}

// z = (L D L^T)^{-1} r with the FP32 copy of the factor (the schedule choice of Handle::apply_precond)
template <typename Ti>
void Batch::precond32(const Ti *r, Ti *z, const KState *stp) {
    cudaStream_t s = h.stream;
    const size_t v = sizeof(Ti);
    const int n = h.n;
    Ti *y = v32[10].as<Ti>();
    const double fb = (4.0 + v) * h.Lf.nnz + 4.0 * (n + 1) + 2.0 * v * n;
    if (h.push_ok(v)) {
        h.timed(PC_FWD, fb, [&] {
            sweep_push<Ti>(h.Lf, L32.as<Ti>(), SW_FWD_DIV, r, invL32_lev.as<Ti>(), mix_epoch, y, stp, h.err(), s);
        });
        h.timed(PC_BWD, fb + v * n, [&] {
            sweep_push<Ti>(h.Ltb, Lt32.as<Ti>(), SW_BWD_IC, y, D32_lev.as<Ti>(), mix_epoch, z, stp, h.err(), s);
        });
        return;
    }
    if (h.cluster_ok(h.Lf, v, true) && h.cluster_ok(h.Ltb, v, true)) {
        h.timed(PC_FWD, fb, [&] {
            sweep_cluster<Ti>(h.Lf, L32.as<Ti>(), SW_FWD_DIV, r, nullptr, h.use_inv_diag ? invL32_lev.as<Ti>() : nullptr,
                              y, nullptr, stp, h.cl_group, h.err(), s);
        });
        h.timed(PC_BWD, fb + v * n, [&] {
            sweep_cluster<Ti>(h.Ltb, Lt32.as<Ti>(), SW_BWD_IC, nullptr, y, D32_lev.as<Ti>(), z, nullptr, stp,
                              h.cl_group, h.err(), s);
        });
        return;
    }
    // all bits set is the sentinel of every value type
    SSG_CUDA(cudaMemsetAsync(y, 0xFF, v * (size_t)n, s));
    h.timed(PC_FWD, fb, [&] {
        sweep_st<Ti>(h.Lf, L32.as<Ti>(), SW_FWD_DIV, r, nullptr, nullptr, y, nullptr, h.ticket(), h.err(), stp, s,
                     h.swcfg, h.use_inv_diag ? invL32.as<Ti>() : nullptr);
    });
    SSG_CUDA(cudaMemsetAsync(z, 0xFF, v * (size_t)n, s));
    h.timed(PC_BWD, fb + v * n, [&] {
        sweep_st<Ti>(h.Ltb, Lt32.as<Ti>(), SW_BWD_IC, nullptr, y, D32.as<Ti>(), z, nullptr, h.ticket() + 1, h.err(),
                     stp, s, h.swcfg, (const Ti *)nullptr);
    });
}

template <typename Ti>
void Batch::inner_setup() {
    cudaStream_t s = h.stream;
    const int n = h.n;
    BDev B = dev_view();
    const int grid = bgrid(NT);
    Ti *rin = v32[1].as<Ti>(), *p = v32[2].as<Ti>(), *z = v32[3].as<Ti>(), *u = v32[4].as<Ti>(),
       *y = v32[5].as<Ti>();
    if (method == SSG_METHOD_ICCG) {
        precond32<Ti>(rin, z, ctl());
        SSG_CUDA(cudaMemcpyAsync(p, z, sizeof(Ti) * (size_t)n, cudaMemcpyDeviceToDevice, s));
        k_brur0<Ti><<<grid, BT, 0, s>>>(B, rin, z);
        SSG_LAUNCHED();
    } else {
        precond32<Ti>(rin, u, ctl());
        k_bneg<Ti><<<grid, BT, 0, s>>>(B, rin, y);
        SSG_LAUNCHED();
        precond32<Ti>(y, z, ctl());
        SSG_CUDA(cudaMemsetAsync(p, 0, sizeof(Ti) * (size_t)n, s));
    }
}

template <typename T, typename Ti>
void Batch::start_mixed(double alpha, double conv) {
    (void)alpha;
    (void)conv;
    cudaStream_t s = h.stream;
    const int n = h.n;
    const int nnzL = h.Lf.nnz;
    // FP32 copies of A and of the FP64 factor (value arrays keep the 16 padding entries)
    A32.ensure(sizeof(Ti) * (size_t)(h.nnz + 16));
    L32.ensure(sizeof(Ti) * (size_t)(nnzL + 16));
    Lt32.ensure(sizeof(Ti) * (size_t)(nnzL + 16));
    for (DBuf *d : {&invL32, &invL32_lev, &D32, &D32_lev}) d->ensure(sizeof(Ti) * (size_t)(n + 1));
    for (auto &v : v32) v.ensure(sizeof(Ti) * (size_t)(n + 1));
    auto narrow_copy = [&](const DBuf &src, DBuf &dst, size_t count) {
        if (!count) return;
        const int g = (int)std::min<size_t>(div_up((int)std::min<size_t>(count, 1u << 30), 256), 4096);
        k_narrow<T, Ti><<<g, 256, 0, s>>>(count, src.as<T>(), dst.as<Ti>());
        SSG_LAUNCHED();
    };
    h.timed(PC_VEC, (double)(sizeof(T) + sizeof(Ti)) * (h.nnz + 2.0 * nnzL + 4.0 * n), [&] {
        narrow_copy(h.A_val, A32, (size_t)h.nnz);
        narrow_copy(h.Lval, L32, (size_t)nnzL);
        narrow_copy(h.Ltval, Lt32, (size_t)nnzL);
        narrow_copy(h.invL, invL32, (size_t)n);
        narrow_copy(h.invL_lev, invL32_lev, (size_t)n);
        narrow_copy(h.Dvec, D32, (size_t)n);
        narrow_copy(h.D_lev, D32_lev, (size_t)n);
    });
    ++mix_epoch;
    BDev B = dev_view();
    k_bmix_begin<<<1, BT, 0, s>>>(B, d_ost.as<OState>(), octl(), eff_inner_tol(), max_ite);
    SSG_LAUNCHED();
    BDev Bo = outer_view();
    const int grid = bgrid(NT);
    k_bscale<T, Ti><<<grid, BT, 0, s>>>(Bo, d_ost.as<OState>(), h.vec[1].as<T>(), v32[1].as<Ti>(), v32[0].as<Ti>());
    SSG_LAUNCHED();
    inner_setup<Ti>();
}

template <typename T, typename Ti>
void Batch::queue_inner(int todo) {
    cudaStream_t s = h.stream;
    const int n = h.n;
    BDev B = dev_view();
    const int grid = bgrid(NT);
    const int *rp = h.A_rp.as<int>(), *ci = h.A_ci.as<int>();
    const Ti *aval = A32.as<Ti>();
    Ti *d = v32[0].as<Ti>(), *r = v32[1].as<Ti>(), *p = v32[2].as<Ti>(), *z = v32[3].as<Ti>(), *u = v32[4].as<Ti>();
    Ti *y = v32[5].as<Ti>(), *v = v32[6].as<Ti>(), *w = v32[7].as<Ti>();
    todo = std::min(todo, max_ite - queued);
    const double nv = (double)sizeof(Ti) * n;
    const double spmv_bytes = (4.0 + sizeof(Ti)) * h.nnz + 4.0 * (n + 1) + 2.0 * nv;
    run_iterations(todo, [&] {
        h.prof.iter = ++iter_no;
        h.prof.pre = true;
        if (method == SSG_METHOD_ICCG) {
            h.timed(PC_SPMV, spmv_bytes, [&] {
                k_bspmv<Ti, true><<<grid, BT, 0, s>>>(B, rp, ci, aval, p, v);
                SSG_LAUNCHED();
            });
            h.timed(PC_VEC, 6 * nv, [&] {
                k_biccg_update<Ti><<<grid, BT, 0, s>>>(B, d, r, p, v);
                SSG_LAUNCHED();
            });
            precond32<Ti>(r, z, ctl());
            h.timed(PC_VEC, 2 * nv, [&] {
                k_biccg_beta<Ti><<<grid, BT, 0, s>>>(B, r, z);
                SSG_LAUNCHED();
            });
            h.timed(PC_VEC, 3 * nv, [&] {
                k_biccg_p<Ti><<<grid, BT, 0, s>>>(B, p, z);
                SSG_LAUNCHED();
            });
        } else {
            h.timed(PC_SPMV, spmv_bytes, [&] {
                k_bspmv<Ti, false><<<grid, BT, 0, s>>>(B, rp, ci, aval, u, v);
                SSG_LAUNCHED();
            });
            precond32<Ti>(v, w, ctl());
            h.timed(PC_VEC, 4 * nv, [&] {
                k_bmrtr_dots<Ti><<<grid, BT, 0, s>>>(B, w, r, v, y);
                SSG_LAUNCHED();
            });
            h.timed(PC_VEC, 10 * nv, [&] {
                k_bmrtr_update<Ti><<<grid, BT, 0, s>>>(B, p, u, d, y, v, r);
                SSG_LAUNCHED();
            });
            h.timed(PC_VEC, 5 * nv, [&] {
                k_bmrtr_zu<Ti><<<grid, BT, 0, s>>>(B, z, w, u);
                SSG_LAUNCHED();
            });
        }
    });
    queued += todo;
    chunk = std::min(chunk * 2, 32);
    SSG_CUDA(cudaMemcpyAsync(h_ctl, ctl(), sizeof(KState), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaMemcpyAsync(h_octl, octl(), sizeof(KState), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaMemcpyAsync(h_st, d_st.p, sizeof(KState) * (size_t)S, cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaMemcpyAsync(h_ost, d_ost.p, sizeof(OState) * (size_t)S, cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaEventRecord(ev_chunk, s));
}

template <typename T, typename Ti>
void Batch::queue_outer_step() {
    cudaStream_t s = h.stream;
    BDev Bo = outer_view();
    const int grid = bgrid(NT);
    OState *O = d_ost.as<OState>();
    T *b = h.vec[0].as<T>(), *r = h.vec[1].as<T>(), *v = h.vec[6].as<T>(), *x = h.vec[8].as<T>();
    const double nv = (double)sizeof(T) * h.n;
    h.timed(PC_VEC, 2 * nv + (double)sizeof(Ti) * h.n, [&] {
        k_bouter_update<T, Ti><<<grid, BT, 0, s>>>(Bo, O, x, v32[0].as<Ti>());
        SSG_LAUNCHED();
    });
    h.timed(PC_SPMV, (4.0 + sizeof(T)) * h.nnz + 4.0 * (h.n + 1) + 2.0 * nv, [&] {
        k_bspmv<T, false><<<grid, BT, 0, s>>>(Bo, h.A_rp.as<int>(), h.A_ci.as<int>(), h.A_val.as<T>(), x, v);
        SSG_LAUNCHED();
    });
    h.timed(PC_VEC, 3 * nv, [&] {
        k_bresid<T><<<grid, BT, 0, s>>>(Bo, O, ctl(), b, v, r, conv_cri, max_ite, eff_inner_tol());
        SSG_LAUNCHED();
    });
    k_bscale<T, Ti><<<grid, BT, 0, s>>>(Bo, O, r, v32[1].as<Ti>(), v32[0].as<Ti>());
    SSG_LAUNCHED();
    inner_setup<Ti>();
}

bool batch_takes(const ssg_options &o, int method) {
    return !o.is_diag_scale && !(method == SSG_METHOD_MRTR && o.precondition_type != 0) && o.accel_factor > 0.0 &&
           o.is_init && o.conv_normalize_type == 0;
}

int solve_batched(Handle &h, Batch *&mb, uint64_t &mver, uint64_t &mpat, int precision, int method, double conv,
                  int max_ite, int nrhs, const void *d_B, void *d_X, int *iters, int *status) {
    const ssg_options &o = h.opt;
    if (h.vtype < 0) throw Error{SSG_ERR_STATE, "no matrix set"};
    if (h.n == 0 || nrhs == 0) {
        for (int j = 0; j < nrhs; ++j) {
            if (iters) iters[j] = 0;
            if (status) status[j] = SSG_OK;
        }
        h.iters = 0;
        h.residual_log.clear();
        return SSG_OK;
    }
    if (!mb) mb = new Batch(h.device);
    mb->h.prof.on = h.prof.on;  // profiling and the sweep schedule follow the owning handle
    // lanes a row: one right-hand side runs the one-system schedule (the cluster sweep is
    // fastest with 4 lanes for real rows; complex rows carry four times the multiply-adds
    // and keep 8); several make the levels wide, and rows of more than 6 off-diagonal
    // entries then run faster on 16 lanes
    int g = h.batch_group;
    if (!g) g = nrhs == 1 ? (h.vtype == SSG_COMPLEX ? 8 : 4) : ((h.nnz - h.n) > 12ll * h.n ? 16 : 8);
    mb->h.swcfg.group = mb->h.cl_group = g;
    mb->h.swcfg.cta_per_sm = h.swcfg.cta_per_sm;
    mb->h.sweep_mode = h.sweep_mode;
    // a handle's own batch (mixed precision, several right-hand sides) serves one matrix:
    // its automatic mode may take the push sweep, as the handle's single solves do
    mb->h.push_auto = true;
    if (mb->h.spin_limit_us != h.spin_limit_us) mb->h.set_spin_limit(h.spin_limit_us);
    AllocStream as(mb->h.stream);  // the batch's buffers are ordered on its own stream
    const int w = h.vtype == SSG_COMPLEX ? 2 : 1;
    const bool same_rhs = !mb->sys.empty() && mb->sys[0].nrhs == nrhs;
    if (mver != h.version && mpat == h.pattern_id && mb->assembled && same_rhs && mb->vtype == h.vtype) {
        // values-only update: the batch keeps its pattern analysis
        SSG_CUDA(cudaStreamSynchronize(h.stream));
        mb->update_values_device(0, h.A_val.p);
        mver = h.version;
    }
    if (mver != h.version || !same_rhs) {
        // the handle's matrix, through the host once per matrix version
        std::vector<int> rp((size_t)h.n + 1), ci((size_t)h.nnz);
        std::vector<double> val((size_t)w * h.nnz), B((size_t)w * h.n * nrhs, 0.0);
        SSG_CUDA(cudaMemcpyAsync(rp.data(), h.A_rp.p, sizeof(int) * rp.size(), cudaMemcpyDeviceToHost, h.stream));
        SSG_CUDA(cudaMemcpyAsync(ci.data(), h.A_ci.p, sizeof(int) * ci.size(), cudaMemcpyDeviceToHost, h.stream));
        SSG_CUDA(cudaMemcpyAsync(val.data(), h.A_val.p, sizeof(double) * val.size(), cudaMemcpyDeviceToHost, h.stream));
        SSG_CUDA(cudaStreamSynchronize(h.stream));
        mb->clear();
        mb->add(h.n, h.nnz, rp.data(), ci.data(), val.data(), h.vtype, nrhs, B.data());
        mver = h.version;
        mpat = h.pattern_id;
    }
    SSG_CUDA(cudaStreamSynchronize(h.stream));  // d_B may come from work queued on the handle's stream
    mb->precision = precision;
    mb->set_rhs_device(0, d_B);
    if (h.vtype == SSG_COMPLEX)
        mb->start<cplx>(method, o.accel_factor, conv, max_ite);
    else
        mb->start<double>(method, o.accel_factor, conv, max_ite);
    mb->wait();
    mb->result_device(0, d_X);
    std::vector<int> it((size_t)nrhs, 0), stt((size_t)nrhs, 0);
    const int rc = mb->result(0, nullptr, it.data(), stt.data());
    for (int j = 0; j < nrhs; ++j) {
        if (iters) iters[j] = it[j];
        if (status) status[j] = stt[j] == ST_CONVERGED ? SSG_OK : SSG_NOT_CONVERGED;
    }
    h.iters = it[nrhs - 1];
    h.alpha_used = o.accel_factor;
    h.residual_log.clear();
    if (o.is_save_residual_log) {
        int len = 0;
        mb->residual_log(0, nrhs - 1, nullptr, 0, &len);
        h.residual_log.resize((size_t)len);
        if (len) mb->residual_log(0, nrhs - 1, h.residual_log.data(), len, &len);
    }
    h.t_setup_ms = mb->t_ms.size() > 0 ? mb->t_ms[0] : 0.0;
    h.t_iter_ms = mb->t_ms.size() > 1 ? mb->t_ms[1] : 0.0;
    return rc;
}

int solve_mixed(Handle &h, Batch *&mb, uint64_t &mver, uint64_t &mpat, int method, double conv, int max_ite,
                const void *d_b, void *d_x) {
    if (!batch_takes(h.opt, method))
        throw Error{SSG_ERR_ARG,
                    "mixed precision solves ICCG or IC-MRTR with a fixed accel_factor > 0, x0 = 0, the |b| "
                    "normaliser and no diagonal scaling"};
    return solve_batched(h, mb, mver, mpat, SSG_PREC_MIXED, method, conv, max_ite, 1, d_b, d_x, nullptr, nullptr);
}

template void Batch::start<double>(int, double, double, int);
template void Batch::start<cplx>(int, double, double, int);

}  // namespace ssg
