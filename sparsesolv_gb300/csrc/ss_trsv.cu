// ss_trsv.cu -- sync-free, level-ordered triangular sweeps.
//
// Restates the substitutions of MatSolverBase (src/MatSolverBase.cpp):
//   forward  (IC_frbc_process :181-189, fr_process :243-278)
//            out_i = (rhs_i - sum_{j<i} L_ij out_j) / L_ii      diagonal last
//   backward (IC_frbc_process :190-199)
//            out_i = D_i * (0 - sum_{j>i} Lt_ij out_j) + aux_i  diagonal first
//   backward (bc_process :291-327)
//            out_i = (rhs_i - sum_{j>i} U_ij out_j) / U_ii     diagonal first
//   Eisenstat (MatSolverMRTR_SGSver.cpp:187-189) fused into one forward sweep:
//            y_i = (rhs_i - aux_i - sum_{j<i} C_ij y_j) / C_ii,  out2_i = y_i + aux_i
//
// Schedule. Rows are streamed in level order (the level-ordered copy of the
// triangle keeps each row's entries contiguous, in their original order). A
// CTA claims a run of consecutive positions with one atomic ticket; a group of
// G lanes owns one row, loads its entries, waits for each dependency to lose
// its sentinel, reduces, and publishes the row's value by overwriting its own
// sentinel. Everything a row waits on was claimed by an earlier ticket, so
// every wait ends; each is also bounded in time and reports ERR_TIMEOUT.
#include "ss_internal.cuh"
#include "ss_krylov.cuh"

namespace ssg {

template <typename T>
struct Ready;
template <>
struct Ready<double> {
    __device__ static bool ok(const double *p, double &v) {
        v = ld_vol(p);
        return !is_sent(v);
    }
    __device__ static void publish(double *p, double v) { st_vol(p, unsent(v)); }
    __device__ static double nan() { return __longlong_as_double(0x7FF8000000000001ll); }
};
template <>
struct Ready<float> {
    __device__ static bool ok(const float *p, float &v) {
        v = ld_vol(p);
        return !is_sent(v);
    }
    __device__ static void publish(float *p, float v) { st_vol(p, unsent(v)); }
    __device__ static float nan() { return __uint_as_float(0x7FC00001u); }
};
template <>
struct Ready<cplx> {
    // both halves must have lost the sentinel (each half is single-copy atomic)
    __device__ static bool ok(const cplx *p, cplx &v) {
        v.x = ld_vol(&p->x);
        v.y = ld_vol(&p->y);
        return !is_sent(v.x) && !is_sent(v.y);
    }
    __device__ static void publish(cplx *p, cplx v) {
        st_vol(&p->y, unsent(v.y));
        st_vol(&p->x, unsent(v.x));
    }
    __device__ static cplx nan() { return {Ready<double>::nan(), Ready<double>::nan()}; }
};
template <>
struct Ready<cplxf> {
    __device__ static bool ok(const cplxf *p, cplxf &v) {
        v.x = ld_vol(&p->x);
        v.y = ld_vol(&p->y);
        return !is_sent(v.x) && !is_sent(v.y);
    }
    __device__ static void publish(cplxf *p, cplxf v) {
        st_vol(&p->y, unsent(v.y));
        st_vol(&p->x, unsent(v.x));
    }
    __device__ static cplxf nan() { return {Ready<float>::nan(), Ready<float>::nan()}; }
};

template <typename T>
__device__ __forceinline__ T wait_value(const T *p, int *err, int backoff_ns) {
    T v;
    if (Ready<T>::ok(p, v)) return v;
    const unsigned long long start = gtimer();
    int polls = 0;
    while (!Ready<T>::ok(p, v)) {
        if (backoff_ns) __nanosleep(backoff_ns);
        if ((++polls & 31) == 0) {
            if (*(volatile int *)err) return Ready<T>::nan();
            if (gtimer() - start > spin_limit_ns(err)) {
                atomicExch(err, ERR_TIMEOUT);
                return Ready<T>::nan();
            }
        }
    }
    return v;
}

constexpr int SW_THREADS = 128;

template <typename T, int G, int MODE>
__global__ void __launch_bounds__(SW_THREADS) k_sweep(int n, const int *__restrict__ perm, const int *__restrict__ prp,
                                                      const int *__restrict__ pci, const T *__restrict__ val,
                                                      const T *rhs, const T *aux, const T *D, T *out, T *out2,
                                                      int *ticket, int *err, const KState *st, const T *dinv,
                                                      int backoff_ns, const int *row_inst, const int *act,
                                                      int act_stride) {
    if (st && !st->active) return;
    constexpr int ROWS = SW_THREADS / G;
    __shared__ int s_base;
    const int g = threadIdx.x / G;
    const int gl = threadIdx.x % G;
    // the value vector the sweep polls: the forward result (y) for FWD_EIS, out otherwise
    T *poll = out;
    for (;;) {
        if (threadIdx.x == 0) s_base = atomicAdd(ticket, ROWS);
        __syncthreads();
        const int base = s_base;
        __syncthreads();
        if (base >= n) return;
        const int t = base + g;
        const int r = t < n ? perm[t] : 0;
        // a batch skips the rows of instances that have ended (nothing of another instance reads them)
        if (t < n && (!row_inst || act[(size_t)row_inst[r] * act_stride])) {
            const int a = prp[t], e = prp[t + 1];
            const bool fwd = (MODE == SW_FWD_DIV || MODE == SW_FWD_EIS);
            const int ob = fwd ? a : a + 1;       // off-diagonal range (empty when the row is)
            const int oe = fwd ? (e > a ? e - 1 : a) : e;
            const int dpos = fwd ? e - 1 : a;     // diagonal position
            // IC pair: the sum is taken negated, and the forward right-hand side starts
            // lane 0's sum, so the row's result is one operation after the reduction
            constexpr bool neg = (MODE == SW_FWD_DIV || MODE == SW_BWD_IC);
            T acc = (MODE == SW_FWD_DIV && gl == 0) ? rhs[r] : Sc<T>::zero();
            for (int k = ob + gl; k < oe; k += G) {
                const int c = pci[k];
                const T v = val[k];
                const T x = wait_value(poll + c, err, backoff_ns);
                acc = madd(acc, neg ? -v : v, x);
            }
            const unsigned gm = group_mask(G);
#pragma unroll
            for (int m = G / 2; m >= 1; m >>= 1) acc = acc + gshfl_xor(acc, m, gm);
            if (gl == 0) {
                // an empty row has no divisor: the result becomes inf/NaN, never an out-of-row read.
                // With dinv the division by the diagonal is a multiplication by its
                // precomputed reciprocal (off the critical path; rounding within 1 ulp).
                T res;
                if (MODE == SW_BWD_IC) {
                    res = madd(aux[r], D[r], acc);  // aux + D * (-sum)
                } else if (MODE == SW_FWD_DIV) {
                    res = dinv ? acc * dinv[r] : acc / ((e > a) ? val[dpos] : Sc<T>::zero());
                } else {
                    T num = rhs[r] - acc;
                    T u = Sc<T>::zero();
                    if (MODE == SW_FWD_EIS) {
                        u = aux[r];
                        num = (rhs[r] - u) - acc;
                    }
                    if (dinv) res = num * dinv[r];
                    else res = num / ((e > a) ? val[dpos] : Sc<T>::zero());
                    if (MODE == SW_FWD_EIS) out2[r] = res + u;
                }
                Ready<T>::publish(out + r, res);
            }
        }
    }
}

template <typename T, int G>
static void launch_sweep(const Tri &tri, const T *val, int mode, const T *rhs, const T *aux, const T *D, T *out,
                         T *out2, int *ticket, int *err, const KState *st, int grid, const T *dinv,
                         const SweepCfg &cfg, cudaStream_t s) {
    const int *perm = tri.perm.as<int>(), *prp = tri.prp.as<int>(), *pci = tri.pci.as<int>();
#define SSG_SW(M)                                                                                                 \
    k_sweep<T, G, M><<<grid, SW_THREADS, 0, s>>>(tri.n, perm, prp, pci, val, rhs, aux, D, out, out2, ticket, err, \
                                                 st, dinv, cfg.backoff_ns, cfg.row_inst, cfg.act, cfg.act_stride)
    switch (mode) {
        case SW_FWD_DIV: SSG_SW(SW_FWD_DIV); break;
        case SW_BWD_IC: SSG_SW(SW_BWD_IC); break;
        case SW_BWD_DIV: SSG_SW(SW_BWD_DIV); break;
        default: SSG_SW(SW_FWD_EIS); break;
    }
#undef SSG_SW
}

static int sweep_grid(int n, int rows_per_cta, int cta_per_sm) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const int want = div_up(n, rows_per_cta);
    const int cap = sms * (cta_per_sm > 0 ? cta_per_sm : 8);
    return want < cap ? want : cap;
}

// group width from the mean off-diagonal count of the triangle
int sweep_group(const Tri &tri) {
    const double mean = tri.n ? (double)(tri.nnz - tri.n) / tri.n : 0.0;
    if (mean <= 6.0) return 8;
    if (mean <= 24.0) return 16;
    return 32;
}

template <typename T>
void sweep_st(const Tri &tri, const T *val, int mode, const T *rhs, const T *aux, const T *D, T *out, T *out2,
              int *d_ticket, int *d_err, const KState *st, cudaStream_t s, const SweepCfg &cfg, const T *dinv) {
    if (tri.n == 0) return;
    SSG_CUDA(cudaMemsetAsync(d_ticket, 0, sizeof(int), s));
    const int G = cfg.group ? cfg.group : sweep_group(tri);
    int cps = cfg.cta_per_sm;
    if (cps <= 0) {
        // rows in flight from the mean level width: two CTAs per SM (4,864 rows at
        // G = 8) keep levels of about a thousand rows busy with the least polling;
        // wide levels (batches of many systems) need more rows in flight
        const double width = tri.nlev > 0 ? (double)tri.n / tri.nlev : (double)tri.n;
        cps = width <= 1024.0 ? 2 : (width >= 8192.0 ? 16 : (int)(width / 512.0));
    }
    const int grid = sweep_grid(tri.n, SW_THREADS / G, cps);
    if (G == 8)
        launch_sweep<T, 8>(tri, val, mode, rhs, aux, D, out, out2, d_ticket, d_err, st, grid, dinv, cfg, s);
    else if (G == 16)
        launch_sweep<T, 16>(tri, val, mode, rhs, aux, D, out, out2, d_ticket, d_err, st, grid, dinv, cfg, s);
    else if (G == 4)
        launch_sweep<T, 4>(tri, val, mode, rhs, aux, D, out, out2, d_ticket, d_err, st, grid, dinv, cfg, s);
    else
        launch_sweep<T, 32>(tri, val, mode, rhs, aux, D, out, out2, d_ticket, d_err, st, grid, dinv, cfg, s);
    SSG_LAUNCHED();
}

template <typename T>
void sweep(const Tri &tri, const T *val, int mode, const T *rhs, const T *aux, const T *D, T *out, T *out2,
           int *d_ticket, int *d_err, cudaStream_t s) {
    sweep_st<T>(tri, val, mode, rhs, aux, D, out, out2, d_ticket, d_err, nullptr, s, SweepCfg{}, nullptr);
}

// reciprocal of each row's diagonal (last entry for a forward triangle, first for a backward one)
template <typename T>
__global__ void k_inv_diag(int n, const int *perm, const int *prp, const T *val, int fwd, T *inv) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int a = prp[t], e = prp[t + 1];
    const T d = (e > a) ? val[fwd ? e - 1 : a] : Sc<T>::zero();
    inv[perm[t]] = Sc<T>::one() / d;
}

template <typename T>
void inv_diag(const Tri &tri, const T *val, T *inv, cudaStream_t s) {
    if (tri.n == 0) return;
    k_inv_diag<T><<<div_up(tri.n, 256), 256, 0, s>>>(tri.n, tri.perm.as<int>(), tri.prp.as<int>(), val,
                                                      tri.lower ? 1 : 0, inv);
    SSG_LAUNCHED();
}

#define SSG_INST(T)                                                                                               \
    template void sweep<T>(const Tri &, const T *, int, const T *, const T *, const T *, T *, T *, int *, int *,  \
                           cudaStream_t);                                                                         \
    template void inv_diag<T>(const Tri &, const T *, T *, cudaStream_t);                                        \
    template void sweep_st<T>(const Tri &, const T *, int, const T *, const T *, const T *, T *, T *, int *, int *, \
                              const KState *, cudaStream_t, const SweepCfg &, const T *);
SSG_INST(double)
SSG_INST(cplx)
SSG_INST(float)
SSG_INST(cplxf)
#undef SSG_INST

}  // namespace ssg
