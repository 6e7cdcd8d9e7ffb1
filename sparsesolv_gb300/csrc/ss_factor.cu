// ss_factor.cu -- shifted IC(0) factorisation and diagonal scaling on the GPU.
//
// The factor restates SprsPreconditioner::detail::IC_decomp_sub
// (src/SprsPreconditioner.cpp:43-111) on the level-ordered lower triangle:
//   L_ij = a_ij - sum_{k<j, k in row i and row j} L_ik L_jk D_k     (j < i)
//   L_ii = alpha a_ii - sum_{k<i} L_ik^2 D_k
//   D_i  = 1 / L_ii   (1 / DBL_EPSILON when |L_ii| < 1e-12)
// One warp owns a row; the entries of the row are updated in column order
// (each uses the already updated L_ik of the same row), the sums over k are
// warp reductions. Rows are claimed in level order through a ticket, and a
// row waits (bounded) for the rows it reads to publish their "done" flags.
#include <cfloat>
#include <mutex>

#include "sparsesolv_gb300.h"
#include "ss_internal.cuh"

namespace ssg {

constexpr int FAC_MAX_PER_LANE = 8;  // rows of the lower triangle up to 256 entries in registers; longer ones in memory

template <typename T>
__device__ __forceinline__ T ldcg(const T *p) {
    return __ldcg(p);
}
template <>
__device__ __forceinline__ cplx ldcg<cplx>(const cplx *p) {
    const double2 v = __ldcg((const double2 *)p);
    return {v.x, v.y};
}
__device__ __forceinline__ void stcg(double *p, double v) { __stcg(p, v); }
__device__ __forceinline__ void stcg(cplx *p, cplx v) { __stcg((double2 *)p, make_double2(v.x, v.y)); }

// bounded wait until row c of the factor has published its done flag
__device__ __forceinline__ void wait_row_done(const int *done, int c, int *err) {
    const volatile int *f = done + c;
    if (*f != 0) return;
    const unsigned long long start = gtimer();
    int polls = 0;
    while (*f == 0) {
        if ((++polls & 63) == 0) {
            if (*(volatile int *)err) return;
            if (gtimer() - start > spin_limit_ns(err)) {
                atomicExch(err, ERR_TIMEOUT);
                return;
            }
        }
    }
}

// A row longer than the registers of a warp hold (a dense coupling row): the
// same recurrence on the row in place in memory. Entry jj takes the updated
// entries left of it from memory (finished before it: written by lane 0, ordered
// by __syncwarp), and finds the columns shared with row j by binary search in
// the row's sorted columns. The sums over k are warp reductions, as for short rows.
template <typename T>
__device__ void factor_long_row(int i, int a, int m, const int *ipos, const int *prp, const int *pci, T *lval, T *D,
                                const int *done, double alpha, int *err, int lane) {
    for (int k = lane; k < m; k += 32) {
        const int c = pci[a + k];
        if (c < i) wait_row_done(done, c, err);
    }
    __syncwarp();
    __threadfence();
    if (pci[a + m - 1] != i) {  // the last entry must be the diagonal (src/SprsPreconditioner.cpp:88-94)
        if (lane == 0) {
            atomicExch(err, ERR_NO_DIAG);
            D[i] = Sc<T>::one();
        }
        return;
    }
    for (int jj = 0; jj < m - 1; ++jj) {
        const int cj = pci[a + jj];
        const int pj = ipos[cj];
        const int aj = prp[pj], mj = prp[pj + 1] - aj;
        T part = Sc<T>::zero();
        for (int l = lane; l < mj; l += 32) {
            const int cc = ldcg(pci + aj + l);
            if (cc >= cj) continue;  // only entries left of the diagonal of row j
            int lo = 0, hi = jj;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (pci[a + mid] < cc) lo = mid + 1;
                else hi = mid;
            }
            if (lo < jj && pci[a + lo] == cc) part = part + ldcg(lval + a + lo) * ldcg(lval + aj + l) * ldcg(D + cc);
        }
        part = warp_sum(part);
        if (lane == 0) stcg(lval + a + jj, ldcg(lval + a + jj) - part);
        __syncwarp();
    }
    T sq = Sc<T>::zero();
    for (int q = lane; q < m - 1; q += 32) {
        const T v = ldcg(lval + a + q);
        sq = sq + v * v * ldcg(D + pci[a + q]);
    }
    sq = warp_sum(sq);
    if (lane == 0) {
        const T s = ldcg(lval + a + m - 1) * Sc<T>::from(alpha) - sq;
        lval[a + m - 1] = s;
        D[i] = (Sc<T>::absv(s) < 1.0e-12) ? Sc<T>::from(1.0 / DBL_EPSILON) : Sc<T>::one() / s;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_ic_factor(int n, const int *perm, const int *ipos, const int *prp,
                                                   const int *pci, T *lval, T *D, int *done, double alpha,
                                                   int *ticket, int *err, const int *sub) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(ticket, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= n) return;
        if (sub) t = sub[t];
        const int i = perm[t];
        const int a = prp[t], m = prp[t + 1] - a;
        if (m > 32 * FAC_MAX_PER_LANE) {
            factor_long_row<T>(i, a, m, ipos, prp, pci, lval, D, done, alpha, err, lane);
            __syncwarp();
            __threadfence();
            if (lane == 0) *(volatile int *)(done + i) = 1;
            continue;
        }
        int bad = 0;
        if (m < 1) bad = 1;
        int c[FAC_MAX_PER_LANE];
        T v[FAC_MAX_PER_LANE], dk[FAC_MAX_PER_LANE];
        // load the row and wait for every row it depends on (all j < i)
#pragma unroll
        for (int q = 0; q < FAC_MAX_PER_LANE; ++q) {
            const int k = lane + 32 * q;
            c[q] = (!bad && k < m) ? pci[a + k] : INT_MAX;
            v[q] = (!bad && k < m) ? lval[a + k] : Sc<T>::zero();
            dk[q] = Sc<T>::zero();
            if (c[q] < i) {
                const volatile int *f = done + c[q];
                if (*f == 0) {
                    const unsigned long long start = gtimer();
                    int polls = 0;
                    while (*f == 0) {
                        if ((++polls & 63) == 0) {
                            if (*(volatile int *)err) break;
                            if (gtimer() - start > spin_limit_ns(err)) {
                                atomicExch(err, ERR_TIMEOUT);
                                break;
                            }
                        }
                    }
                }
            }
        }
        __syncwarp();
        __threadfence();
#pragma unroll
        for (int q = 0; q < FAC_MAX_PER_LANE; ++q)
            if (c[q] < i) dk[q] = ldcg(D + c[q]);
        // off-diagonal entries in column order
        const int mo = bad ? 0 : m - 1;  // entries before the (expected) diagonal
        for (int jj = 0; jj < mo; ++jj) {
            // column j = c of entry jj (owned by lane jj % 32, slot jj / 32)
            int cj = 0;
            T s = Sc<T>::zero();
#pragma unroll
            for (int q = 0; q < FAC_MAX_PER_LANE; ++q) {
                if (q == jj / 32) {
                    cj = __shfl_sync(0xffffffffu, c[q], jj & 31);
                    s = Sc<T>::shfl(v[q], jj & 31);
                }
            }
            if (cj >= i) break;
            // row j of the factor (final: its done flag was observed above)
            const int pj = ipos[cj];
            const int aj = prp[pj], mj = prp[pj + 1] - aj;
            T part = Sc<T>::zero();
            for (int base = 0; base < mj; base += 32) {
                const int l = base + lane;
                const int cl = l < mj ? ldcg(pci + aj + l) : INT_MAX;
                const T vl = l < mj ? ldcg(lval + aj + l) : Sc<T>::zero();
                const int cnt = min(32, mj - base);
                for (int src = 0; src < cnt; ++src) {
                    const int cc = __shfl_sync(0xffffffffu, cl, src);
                    const T vv = Sc<T>::shfl(vl, src);
                    if (cc >= cj) break;  // uniform: only entries left of the diagonal of row j
#pragma unroll
                    for (int q = 0; q < FAC_MAX_PER_LANE; ++q)
                        if (lane + 32 * q < jj && c[q] == cc) part = part + v[q] * vv * dk[q];
                }
            }
            part = warp_sum(part);
            s = s - part;
#pragma unroll
            for (int q = 0; q < FAC_MAX_PER_LANE; ++q)
                if (lane + 32 * q == jj) v[q] = s;
        }
        // the last entry must be the diagonal (src/SprsPreconditioner.cpp:88-94)
        int last_c = 0;
        T diag = Sc<T>::zero();
        if (!bad) {
#pragma unroll
            for (int q = 0; q < FAC_MAX_PER_LANE; ++q) {
                if (q == (m - 1) / 32) {
                    last_c = __shfl_sync(0xffffffffu, c[q], (m - 1) & 31);
                    diag = Sc<T>::shfl(v[q], (m - 1) & 31);
                }
            }
        }
        if (bad || last_c != i) {
            if (lane == 0) atomicExch(err, (m > 32 * FAC_MAX_PER_LANE) ? ERR_ROW_TOO_LONG : ERR_NO_DIAG);
            if (lane == 0) D[i] = Sc<T>::one();
        } else {
            T sq = Sc<T>::zero();
#pragma unroll
            for (int q = 0; q < FAC_MAX_PER_LANE; ++q)
                if (lane + 32 * q < m - 1 && c[q] < i) sq = sq + v[q] * v[q] * dk[q];
            sq = warp_sum(sq);
            const T s = diag * Sc<T>::from(alpha) - sq;
#pragma unroll
            for (int q = 0; q < FAC_MAX_PER_LANE; ++q)
                if (lane + 32 * q == m - 1) v[q] = s;
            if (lane == 0) D[i] = (Sc<T>::absv(s) < 1.0e-12) ? Sc<T>::from(1.0 / DBL_EPSILON) : Sc<T>::one() / s;
        }
#pragma unroll
        for (int q = 0; q < FAC_MAX_PER_LANE; ++q)
            if (lane + 32 * q < m && !bad) lval[a + lane + 32 * q] = v[q];
        __syncwarp();
        __threadfence();
        if (lane == 0) *(volatile int *)(done + i) = 1;
    }
}

// ---------------------------------------------------------------- fast factor
// Rows of at most 32 entries (the voxel curl-curl matrices have 16 to 18 in
// their lower triangle): lane k owns entry k of row i. The entries are
// finished left to right; as soon as entry kk is final, every lane jj > kk
// subtracts its contribution L_ik L_jk D_k (when column k also appears in
// row j) -- the same terms, subtracted in the same order, as the reference's
// loop over kk, so with FMA contraction off (this file is compiled with
// -fmad=false) the real factor is bit-identical to the reference's. Before a
// lane waits for row j (its entry's column), it stages row j's columns (the
// row's start in the level-ordered arrays comes from a per-entry table built
// once per pattern) and finds where row j holds each earlier column of row i;
// once row j's done flag is seen, only its pivot and those values are loaded.
constexpr int FF_MAXROW = 32;
int factor_blocks_per_sm = 4;  // rows in flight: enough for a level, few enough not to congest L2
template <typename T>
__host__ __device__ constexpr int ff_warps() { return sizeof(T) == 8 ? 3 : 2; }  // static shared memory below 48 KB

// NAT: rows in natural order (perm is the identity, a row's dependencies start
// at prp[c]); dep and perm are then not read.
template <typename T, bool NAT = false>
__global__ void __launch_bounds__(ff_warps<T>() * 32) k_ic_factor_fast(int n, const int *perm, const int *prp,
                                                                       const int *pci, const int2 *dep, T *lval,
                                                                       T *D, int *done, double alpha, int *ticket,
                                                                       int *err, int backoff_ns, const int *sub) {
    constexpr int FF_WARPS = ff_warps<T>();
    __shared__ int s_c[FF_WARPS][FF_MAXROW][FF_MAXROW - 1];            // columns of row j
    __shared__ unsigned char s_p[FF_WARPS][FF_MAXROW][FF_MAXROW - 1];  // step kk: position of c_kk in row j
    __shared__ T s_v[FF_WARPS][FF_MAXROW][FF_MAXROW - 1];              // step kk: L_jk
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(ticket, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= n) return;
        if (!NAT && sub) t = sub[t];
        const int i = NAT ? t : perm[t];
        const int a = prp[t], m = prp[t + 1] - a;
        const bool have = lane < m;
        const int c = have ? pci[a + lane] : INT_MAX;
        T v = have ? lval[a + lane] : Sc<T>::zero();
        const int last_c = __shfl_sync(0xffffffffu, c, (m - 1) & 31);
        // caller-given pattern (natural order): off-diagonal columns must lie in [0, i) and
        // ascend strictly (the merge below walks both rows in column order)
        const int prev_c = __shfl_up_sync(0xffffffffu, c, 1);
        const bool bad_col =
            NAT && __any_sync(0xffffffffu, have && ((lane < m - 1 && (c < 0 || c >= i)) || (lane > 0 && prev_c >= c)));
        if (m < 1 || m > FF_MAXROW || last_c != i || bad_col) {
            // no diagonal last (src/SprsPreconditioner.cpp:88-94), a bad caller pattern, or too long
            if (lane == 0) {
                atomicExch(err, m > FF_MAXROW ? ERR_ROW_TOO_LONG : (bad_col && last_c == i) ? ERR_PATTERN : ERR_NO_DIAG);
                D[i] = Sc<T>::one();
            }
            __syncwarp();
            __threadfence();
            if (lane == 0) *(volatile int *)(done + i) = 1;
            continue;
        }
        const bool off = have && lane < m - 1;  // off-diagonal entry (column < i)
        // Before the wait, from the pattern alone: row j = c (without its diagonal, its last
        // entry) has its columns staged, and each lane finds, for every earlier step kk,
        // whether row j holds column c_kk and where (the merge the step would otherwise walk
        // on the critical path).
        int2 dj = make_int2(0, 0);
        int mj = 0;
        unsigned hits = 0u;  // bit kk: row j holds column c_kk
        if (off) {
            dj = NAT ? make_int2(prp[c], prp[c + 1] - prp[c]) : dep[a + lane];
            mj = min(dj.y - 1, FF_MAXROW - 1);
#pragma unroll
            for (int l = 0; l < FF_MAXROW - 1; ++l)
                if (l < mj) s_c[w][lane][l] = __ldg(pci + dj.x + l);
        }
        {
            int ptr = 0;
            for (int kk = 0; kk < m - 1; ++kk) {
                const int ck = __shfl_sync(0xffffffffu, c, kk);
                if (off && lane > kk) {
                    while (ptr < mj && s_c[w][lane][ptr] < ck) ++ptr;
                    if (ptr < mj && s_c[w][lane][ptr] == ck) {
                        hits |= 1u << kk;
                        s_p[w][lane][kk] = (unsigned char)ptr;
                    }
                }
            }
        }
        T dk = Sc<T>::zero();
        if (off) {
            const volatile int *f = done + c;
            if (*f == 0) {
                const unsigned long long start = gtimer();
                int polls = 0;
                while (*f == 0) {
                    if (backoff_ns) __nanosleep(backoff_ns);
                    if ((++polls & 15) == 0) {
                        if (*(volatile int *)err) break;
                        if (gtimer() - start > spin_limit_ns(err)) {
                            atomicExch(err, ERR_TIMEOUT);
                            break;
                        }
                    }
                }
            }
            __threadfence();
            // row j is final: its pivot and the values this row's steps use
            dk = ldcg(D + c);
            for (unsigned h = hits; h; h &= h - 1) {
                const int kk = __ffs(h) - 1;
                s_v[w][lane][kk] = ldcg(lval + dj.x + s_p[w][lane][kk]);
            }
        }
        __syncwarp();
        // diagonal lane starts from alpha * a_ii (src/SprsPreconditioner.cpp:95)
        if (lane == m - 1) v = v * Sc<T>::from(alpha);
        for (int kk = 0; kk < m - 1; ++kk) {
            const T Lk = Sc<T>::shfl(v, kk);  // final L_ik
            const T Dk = Sc<T>::shfl(dk, kk);
            // an off-diagonal lane subtracts L_ik L_jk D_k when row j holds column k; the
            // diagonal lane L_ik L_ik D_k: one update for both
            const bool diag = lane == m - 1;
            const bool hit = diag || ((hits >> kk) & 1u);
            const T o = diag ? Lk : s_v[w][lane][kk];
            if (hit) v = v - (Lk * o) * Dk;
        }
        if (have) lval[a + lane] = v;
        if (lane == m - 1) D[i] = (Sc<T>::absv(v) < 1.0e-12) ? Sc<T>::from(1.0 / DBL_EPSILON) : Sc<T>::one() / v;
        __syncwarp();
        __threadfence();
        if (lane == 0) *(volatile int *)(done + i) = 1;
    }
}

__global__ void k_dep_starts(int nnz, const int *pci, const int *ipos, const int *prp, int2 *dep) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnz) return;
    const int p = ipos[pci[k]];
    dep[k] = make_int2(prp[p], prp[p + 1] - prp[p]);
}

__global__ void k_max_rowlen(int n, const int *prp, int *out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) atomicMax(out, prp[t + 1] - prp[t]);
}

void factor_plan(const Tri &L, DBuf &dep, int &max_row, cudaStream_t s) {
    dep.ensure(sizeof(int2) * (size_t)(L.nnz + 1));
    max_row = 0;
    if (L.n == 0) return;
    k_dep_starts<<<div_up(L.nnz, 256), 256, 0, s>>>(L.nnz, L.pci.as<int>(), L.ipos.as<int>(), L.prp.as<int>(),
                                                    dep.as<int2>());
    SSG_LAUNCHED();
    DBuf mx;
    mx.alloc(sizeof(int));
    SSG_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(int), s));
    k_max_rowlen<<<div_up(L.n, 256), 256, 0, s>>>(L.n, L.prp.as<int>(), mx.as<int>());
    SSG_LAUNCHED();
    SSG_CUDA(cudaMemcpyAsync(&max_row, mx.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaStreamSynchronize(s));
}

template <typename T>
void ic_factor(const Tri &L, T *lval, T *D, double alpha, int *d_err, int *d_ticket, cudaStream_t s,
               const int2 *dep, int max_row, int *done, int backoff_ns, const int *sub, int nsub) {
    if (L.n == 0) return;
    const int cnt = sub ? nsub : L.n;  // rows to factor (sub: their level-ordered positions, ascending)
    if (cnt == 0) return;
    SSG_CUDA(cudaMemsetAsync(done, 0, sizeof(int) * (size_t)L.n, s));
    SSG_CUDA(cudaMemsetAsync(d_ticket, 0, sizeof(int), s));
    int dev = 0, sms = 0;
    SSG_CUDA(cudaGetDevice(&dev));
    SSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (dep && max_row <= FF_MAXROW) {
        constexpr int W = ff_warps<T>();
        // wide levels (batches of many systems) keep more rows in flight
        const double width = L.nlev > 0 ? (double)cnt / L.nlev : (double)cnt;
        const int per_sm = width >= 8192.0 ? 6 : factor_blocks_per_sm;
        const int blocks = min(div_up(cnt, W), sms * per_sm);
        k_ic_factor_fast<T><<<blocks, W * 32, 0, s>>>(cnt, L.perm.as<int>(), L.prp.as<int>(), L.pci.as<int>(), dep,
                                                      lval, D, done, alpha, d_ticket, d_err, backoff_ns, sub);
    } else {
        const int warps = min(cnt, sms * 32);
        k_ic_factor<T><<<div_up(warps * 32, 256), 256, 0, s>>>(cnt, L.perm.as<int>(), L.ipos.as<int>(),
                                                               L.prp.as<int>(), L.pci.as<int>(), lval, D, done,
                                                               alpha, d_ticket, d_err, sub);
    }
    SSG_LAUNCHED();
}

// Rows whose factor equals another row's (a system repeated in a batch, once per
// right-hand side): copy that row's entries and pivot instead of factoring it.
// rep_src[i] = the source row of row i, or -1; both rows have the same pattern.
template <typename T>
__global__ void k_copy_replica_rows(int n, const int *rep_src, const int *ipos, const int *prp, T *lval, T *D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int src = rep_src[i];
    if (src < 0) return;
    const int pd = prp[ipos[i]], ps = prp[ipos[src]], m = prp[ipos[i] + 1] - pd;
    for (int k = 0; k < m; ++k) lval[pd + k] = lval[ps + k];
    D[i] = D[src];
}

template <typename T>
void copy_replica_rows(const Tri &L, const int *rep_src, T *lval, T *D, cudaStream_t s) {
    if (L.n == 0) return;
    k_copy_replica_rows<T><<<div_up(L.n, 256), 256, 0, s>>>(L.n, rep_src, L.ipos.as<int>(), L.prp.as<int>(), lval, D);
    SSG_LAUNCHED();
}

// level-ordered positions t of the rows without a source (rep_src[perm[t]] < 0), ascending
__global__ void k_own_flags(int n, const int *perm, const int *rep_src, int *flag) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) flag[t] = rep_src[perm[t]] < 0 ? 1 : 0;
}
__global__ void k_own_scatter(int n, const int *perm, const int *rep_src, const int *pos, int *sub) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n && rep_src[perm[t]] < 0) sub[pos[t]] = t;
}

int own_rows(const Tri &L, const int *rep_src, DBuf &sub, cudaStream_t s) {
    if (L.n == 0) return 0;
    DBuf pos, tot, tmp;
    pos.alloc(sizeof(int) * ((size_t)L.n + 1));
    tot.alloc(sizeof(int));
    k_own_flags<<<div_up(L.n, 256), 256, 0, s>>>(L.n, L.perm.as<int>(), rep_src, pos.as<int>());
    SSG_LAUNCHED();
    scan_exclusive(pos.as<int>(), L.n, tot.as<int>(), s, tmp);
    int cnt = 0;
    SSG_CUDA(cudaMemcpyAsync(&cnt, tot.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaStreamSynchronize(s));
    sub.ensure(sizeof(int) * ((size_t)cnt + 1));
    k_own_scatter<<<div_up(L.n, 256), 256, 0, s>>>(L.n, L.perm.as<int>(), rep_src, pos.as<int>(), sub.as<int>());
    SSG_LAUNCHED();
    SSG_CUDA(cudaStreamSynchronize(s));
    return cnt;
}

// ---------------------------------------------------------------- diagonal scaling
// SprsPreconditioner::DiagScaling (src/SprsPreconditioner.cpp:150-231):
// d_i = 1/sqrt(|a_ii|) for real, 1/sqrt(std::norm(a_ii)) = 1/|a_ii| for complex
// (the reference's quirk, kept), 1/DBL_EPSILON when the root is < 1e-12.
template <typename T>
__global__ void k_diag_scaling(int n, const int *rp, const int *ci, const T *val, const T *b, T *d, T *bs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
        if (ci[k] == i) {
            const double t1 = Sc<T>::is_complex ? Sc<T>::abs2(val[k]) : Sc<T>::absv(val[k]);
            const double t1b = sqrt(t1);
            const double t2 = (t1b < 1.0e-12) ? 1.0 / DBL_EPSILON : 1.0 / t1b;
            d[i] = Sc<T>::from(t2);
            if (b) bs[i] = b[i] * Sc<T>::from(t2);
            return;
        }
    }
    d[i] = Sc<T>::zero();
    if (b) bs[i] = Sc<T>::zero();
}

// D A D: MatSolverBase::makeDiagMatTrans (src/MatSolverBase.cpp:99-141)
template <typename T>
__global__ void k_dad(int n, const int *rp, const int *ci, const T *val, const T *d, T *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const T di = d[i];
    for (int k = rp[i]; k < rp[i + 1]; ++k) out[k] = val[k] * (di * d[ci[k]]);
}

template <typename T>
__global__ void k_pivots_positive(int n, const T *D, int *flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && !(Sc<T>::re(D[i]) > 0.0)) atomicExch(flag, 0);
}

template <typename T>
void diag_scaling(int n, const int *rp, const int *ci, const T *val, const T *b, T *d, T *bs, cudaStream_t s) {
    if (n == 0) return;
    k_diag_scaling<T><<<div_up(n, 256), 256, 0, s>>>(n, rp, ci, val, b, d, bs);
    SSG_LAUNCHED();
}
template <typename T>
void dad_values(int n, const int *rp, const int *ci, const T *val, const T *d, T *out, cudaStream_t s) {
    if (n == 0) return;
    k_dad<T><<<div_up(n, 256), 256, 0, s>>>(n, rp, ci, val, d, out);
    SSG_LAUNCHED();
}
template <typename T>
void all_pivots_positive(int n, const T *D, int *d_flag, cudaStream_t s) {
    SSG_CUDA(cudaMemsetAsync(d_flag, 0, sizeof(int), s));
    const int one = 1;
    SSG_CUDA(cudaMemcpyAsync(d_flag, &one, sizeof(int), cudaMemcpyHostToDevice, s));
    if (n > 0) {
        k_pivots_positive<T><<<div_up(n, 256), 256, 0, s>>>(n, D, d_flag);
        SSG_LAUNCHED();
    }
}

#define SSG_INST(T)                                                                                      \
    template void ic_factor<T>(const Tri &, T *, T *, double, int *, int *, cudaStream_t, const int2 *, int,  \
                               int *, int, const int *, int);                                                \
    template void copy_replica_rows<T>(const Tri &, const int *, T *, T *, cudaStream_t);                     \
    template void diag_scaling<T>(int, const int *, const int *, const T *, const T *, T *, T *,        \
                                  cudaStream_t);                                                         \
    template void dad_values<T>(int, const int *, const int *, const T *, const T *, T *, cudaStream_t); \
    template void all_pivots_positive<T>(int, const T *, int *, cudaStream_t);
SSG_INST(double)
SSG_INST(cplx)
#undef SSG_INST

// ---------------------------------------------------------------- factor without allocation
// For callers that may not allocate device memory (ssg_ic_factor_noalloc): the
// row flags, the row ticket and the error word live in one file-scope array
// that every device loading this library holds until the process exits.
// Layout: [0] ticket, [1] error code, [NA_HEAD, NA_HEAD + n) row done flags.
constexpr int NA_HEAD = 64;  // 256 bytes, keeps the flags 256-byte aligned
static __device__ __align__(256) int g_noalloc_scratch[NA_HEAD + SSG_NOALLOC_MAX_ROWS];

// Device address of the scratch array on device `dev`, which must be current.
// The array's name in host code is only a stand-in; a kernel needs this
// address. Looked up once per device and kept.
static int noalloc_scratch(int dev, int **out) {
    constexpr int MAX_DEV = 64;
    static std::mutex mu;
    static int *addr[MAX_DEV] = {};
    if (dev < 0 || dev >= MAX_DEV) return SSG_ERR_ARG;
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return SSG_ERR_CUDA;
        addr[dev] = (int *)p;
    }
    *out = addr[dev];
    return SSG_OK;
}

template <typename T>
static cudaError_t noalloc_launch(int n, const int *lrp, const int *lci, void *lval, void *D, double alpha,
                                  int *scr, int sms, cudaStream_t s) {
    constexpr int W = ff_warps<T>();
    const int blocks = min(div_up(n, W), sms * factor_blocks_per_sm);
    k_ic_factor_fast<T, true><<<blocks, W * 32, 0, s>>>(n, nullptr, lrp, lci, nullptr, (T *)lval, (T *)D,
                                                        scr + NA_HEAD, alpha, scr, scr + 1, 0, nullptr);
    return cudaGetLastError();
}

// Natural-order IC(0) with the scratch above. Every failure returns a code;
// nothing here allocates, host or device, on the way to a result.
static bool aligned_to(const void *p, size_t a) { return ((uintptr_t)p % a) == 0; }

int ic_factor_noalloc(int n, int nnz, const int *lrp, const int *lci, const void *val, void *lval, void *D,
                      double alpha, int vtype, cudaStream_t s) {
    if (n < 0 || nnz < 0 || n > SSG_NOALLOC_MAX_ROWS) return SSG_ERR_ARG;
    if (!(alpha > 0.0) || (vtype != SSG_REAL && vtype != SSG_COMPLEX)) return SSG_ERR_ARG;
    if (n == 0) return SSG_OK;
    if (!lrp || !lci || !val || !lval || !D || nnz < n) return SSG_ERR_ARG;
    // the kernel reads a complex value as one 16-byte load, a real one as 8 bytes
    const size_t va = vtype == SSG_COMPLEX ? 16 : 8;
    if (!aligned_to(lrp, 4) || !aligned_to(lci, 4) || !aligned_to(val, va) || !aligned_to(lval, va) ||
        !aligned_to(D, va))
        return SSG_ERR_ARG;
    // the call reads its error word back and waits for the stream: not inside a capture
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return SSG_ERR_CUDA;
    if (cap != cudaStreamCaptureStatusNone) return SSG_ERR_STATE;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SSG_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return SSG_ERR_CUDA;
    int *scr = nullptr;
    const int rc = noalloc_scratch(dev, &scr);
    if (rc != SSG_OK) return rc;
    const size_t vb = vtype == SSG_COMPLEX ? sizeof(cplx) : sizeof(double);
    if (val != lval && cudaMemcpyAsync(lval, val, vb * (size_t)nnz, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return SSG_ERR_CUDA;
    // the ticket, the error word and the flags of this call's rows start at zero
    if (cudaMemsetAsync(scr, 0, sizeof(int) * (NA_HEAD + (size_t)n), s) != cudaSuccess) return SSG_ERR_CUDA;
    const cudaError_t le = vtype == SSG_COMPLEX ? noalloc_launch<cplx>(n, lrp, lci, lval, D, alpha, scr, sms, s)
                                                : noalloc_launch<double>(n, lrp, lci, lval, D, alpha, scr, sms, s);
    // from here on a failure waits for the queued work first, so the shared scratch is
    // idle when the call returns, whatever the outcome
    auto fail = [&](int code) {
        (void)cudaStreamSynchronize(s);
        return code;
    };
    if (le != cudaSuccess) return fail(SSG_ERR_CUDA);
    try {
        note_launch();
    } catch (...) {
        return fail(SSG_ERR_CUDA);
    }
    int err = 0;
    if (cudaMemcpyAsync(&err, scr + 1, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return fail(SSG_ERR_CUDA);
    if (cudaStreamSynchronize(s) != cudaSuccess) return SSG_ERR_CUDA;
    switch (err) {
        case ERR_NONE: return SSG_OK;
        case ERR_TIMEOUT: return SSG_ERR_TIMEOUT;
        case ERR_NO_DIAG: return SSG_ERR_NO_DIAGONAL;
        default: return SSG_ERR_ARG;  // a row longer than 32 entries, or a bad column pattern
    }
}

}  // namespace ssg
