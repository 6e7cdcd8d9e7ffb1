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

// an instance's tile partials, added in tile order
template <int K>
__device__ __forceinline__ void inst_sum(const BDev &B, int s, double (&tot)[K]) {
#pragma unroll
    for (int k = 0; k < K; ++k) tot[k] = 0.0;
    for (int t = B.sys_tile[s]; t < B.sys_tile[s + 1]; ++t)
#pragma unroll
        for (int k = 0; k < K; ++k) tot[k] += __ldcg(B.part + (size_t)t * BATCH_PARTS + k);
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
        if (!B.st[B.tile_sys[t]].active) continue;
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
// y = A x on the rows of active instances (G = 8 lanes a row, the lanes' sums
// combined by a fixed butterfly); with DOT also alpha = rur0 / (x . y).
template <typename T, bool DOT>
__global__ void __launch_bounds__(BT) k_bspmv(BDev B, const int *__restrict__ rp, const int *__restrict__ ci,
                                              const T *__restrict__ val, const T *__restrict__ x, T *__restrict__ y) {
    if (!B.ctl->active) return;
    constexpr int G = 8, RPB = BT / G;
    const int g = threadIdx.x / G, gl = threadIdx.x % G;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        if (!B.st[B.tile_sys[t]].active) continue;
        const int2 tr = B.tile[t];
        double acc2[2] = {0.0, 0.0};
        for (int row0 = tr.x; row0 < tr.y; row0 += RPB) {
            const int row = row0 + g;
            T acc = Sc<T>::zero();
            if (row < tr.y) {
                const int a = rp[row], e = rp[row + 1];
                for (int k = a + gl; k < e; k += G) acc = acc + val[k] * x[ci[k]];
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
        putS<T>(st->alpha, getS<T>(st->rur0) / getS<T>(tot));
    }
    __syncthreads();
    if (threadIdx.x == 0) *B.counter = 0u;
}

// ---------------------------------------------------------------- ICCG steps
template <typename T>
__global__ void __launch_bounds__(BT) k_biccg_update(BDev B, T *x, T *r, const T *p, const T *ap) {
    if (!B.ctl->active) return;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        const KState *st = B.st + B.tile_sys[t];
        if (!st->active) continue;
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
        if (!B.st[B.tile_sys[t]].active) continue;
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
        const T rur1 = getS<T>(tot);
        putS<T>(st->beta, rur1 / getS<T>(st->rur0));
        putS<T>(st->rur0, rur1);
    }
    __syncthreads();
    if (threadIdx.x == 0) *B.counter = 0u;
}

template <typename T>
__global__ void __launch_bounds__(BT) k_biccg_p(BDev B, T *p, const T *z) {
    if (!B.ctl->active) return;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        const KState *st = B.st + B.tile_sys[t];
        if (!st->active) continue;
        const T beta = getS<T>(st->beta);
        const int2 tr = B.tile[t];
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) p[i] = p[i] * beta + z[i];
    }
}

// ---------------------------------------------------------------- IC-MRTR steps
template <typename T>
__global__ void __launch_bounds__(BT) k_bmrtr_dots(BDev B, const T *a, const T *b, const T *c, const T *y) {
    if (!B.ctl->active) return;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        if (!B.st[B.tile_sys[t]].active) continue;
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
        const T wr = getS<T>(tot + 0), vw = getS<T>(tot + 2), wy = getS<T>(tot + 4);
        for (int k = 0; k < 6; ++k) st->dots[k] = tot[k];
        T zeta, eta, nu = getS<T>(st->nu), zeta_old = getS<T>(st->zeta_old);
        if (st->it == 0) {
            zeta = wr / vw;
            zeta_old = zeta;
            eta = Sc<T>::zero();
        } else {
            const T temp0 = Sc<T>::one() / (nu * vw - wy * wy);
            zeta = nu * wr * temp0;
            eta = (-1.0 * wy) * wr * temp0;
        }
        nu = zeta * wr;
        const T ptemp = eta * zeta_old / zeta;
        zeta_old = zeta;
        putS<T>(st->zeta, zeta);
        putS<T>(st->eta, eta);
        putS<T>(st->nu, nu);
        putS<T>(st->ptemp, ptemp);
        putS<T>(st->zeta_old, zeta_old);
    }
    __syncthreads();
    if (threadIdx.x == 0) *B.counter = 0u;
}

template <typename T>
__global__ void __launch_bounds__(BT) k_bmrtr_update(BDev B, T *p, const T *u, T *x, T *y, const T *v, T *r) {
    if (!B.ctl->active) return;
    for (int t = blockIdx.x; t < B.NT; t += gridDim.x) {
        const KState *st = B.st + B.tile_sys[t];
        if (!st->active) continue;
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
        const KState *st = B.st + B.tile_sys[t];
        if (!st->active) continue;
        const T zeta = getS<T>(st->zeta), eta = getS<T>(st->eta);
        const int2 tr = B.tile[t];
        for (int i = tr.x + threadIdx.x; i < tr.y; i += BT) {
            const T zi = z[i] * eta + zeta * w[i];
            z[i] = zi;
            u[i] = u[i] - zi;
        }
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
    SSG_CUDA(cudaEventCreateWithFlags(&ev_chunk, cudaEventDisableTiming));
    for (auto &e : ev) SSG_CUDA(cudaEventCreate(&e));
}

Batch::~Batch() {
    cudaSetDevice(h.device);
    if (h_st) cudaFreeHost(h_st);
    if (h_ctl) cudaFreeHost(h_ctl);
    if (ev_chunk) cudaEventDestroy(ev_chunk);
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
    long long N = 0, NNZ = 0;
    for (size_t q = 0; q < sys.size(); ++q)
        for (int j = 0; j < sys[q].nrhs; ++j) {
            inst_sys.push_back((int)q);
            inst_rhs.push_back(j);
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
    h.set_matrix((int)N, (int)NNZ, rp.data(), ci.data(), val.data(), vtype, cudaMemcpyHostToDevice);
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
    if (h_st) cudaFreeHost(h_st);
    h_st = nullptr;
    SSG_CUDA(cudaMallocHost((void **)&h_st, sizeof(KState) * (size_t)S));
    if (!h_ctl) SSG_CUDA(cudaMallocHost((void **)&h_ctl, sizeof(KState)));
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
    B.ctl = ctl();
    B.part = d_part.as<double>();
    B.counter = (unsigned *)(d_ctl_counter.as<char>() + sizeof(KState));
    B.logs = d_logs.as<double>();
    B.log_stride = max_ite + 2;
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
    SSG_CUDA(cudaEventRecord(ev[0], s));
    const int n = h.n;
    // the factor is recomputed on every start, as the reference's solve() does
    h.fac_valid = false;
    h.ensure_factor<T>(alpha, false);
    h.ensure_work(sizeof(T));
    d_logs.ensure(sizeof(double) * (size_t)S * (size_t)(max_ite + 2));
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

template <typename T>
void Batch::queue_chunk() {
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
    for (int c = 0; c < todo; ++c) {
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
    }
    queued += todo;
    chunk = std::min(chunk * 2, 32);
    SSG_CUDA(cudaMemcpyAsync(h_ctl, ctl(), sizeof(KState), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaEventRecord(ev_chunk, s));
}

bool Batch::poll() {
    if (!running) return true;
    const cudaError_t q = cudaEventQuery(ev_chunk);
    if (q == cudaErrorNotReady) return false;
    SSG_CUDA(q);
    h.check_err("batched iterations");
    if (h_ctl->active && queued < max_ite) {
        if (vtype == SSG_COMPLEX)
            queue_chunk<cplx>();
        else
            queue_chunk<double>();
        return false;
    }
    cudaStream_t s = h.stream;
    SSG_CUDA(cudaMemcpyAsync(h_st, d_st.p, sizeof(KState) * (size_t)S, cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaEventRecord(ev[2], s));
    SSG_CUDA(cudaStreamSynchronize(s));
    int most = 0;
    for (int q = 0; q < S; ++q) most = std::max(most, h_st[q].it);
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

int Batch::result(int index, double *X, int *iters, int *status) {
    if (running) throw Error{SSG_ERR_STATE, "batch is running"};
    if (index < 0 || index >= (int)sys.size()) throw Error{SSG_ERR_ARG, "bad system index"};
    if (!assembled || t_ms.empty()) throw Error{SSG_ERR_STATE, "no finished solve"};
    const size_t vb = vtype == SSG_COMPLEX ? 16 : 8;
    int rc = SSG_OK;
    for (int q = 0; q < S; ++q) {
        if (inst_sys[q] != index) continue;
        const int j = inst_rhs[q], n = sys[index].n;
        if (X)
            SSG_CUDA(cudaMemcpyAsync((char *)X + vb * (size_t)n * j, h.vec[8].as<char>() + vb * (size_t)inst_row[q],
                                     vb * (size_t)n, cudaMemcpyDeviceToHost, h.stream));
        if (iters) iters[j] = h_st[q].it;
        if (status) status[j] = h_st[q].status;
        if (h_st[q].status != ST_CONVERGED) rc = SSG_NOT_CONVERGED;
    }
    SSG_CUDA(cudaStreamSynchronize(h.stream));
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
    const int len = h_st[q].log_len >= 0 ? h_st[q].log_len : h_st[q].it + 1;
    if (length) *length = len;
    if (out && capacity > 0) {
        const int m = std::min(capacity, len);
        if (m > 0)
            SSG_CUDA(cudaMemcpy(out, d_logs.as<double>() + (size_t)q * (max_ite + 2), sizeof(double) * (size_t)m,
                                cudaMemcpyDeviceToHost));
    }
    return SSG_OK;
}

template void Batch::start<double>(int, double, double, int);
template void Batch::start<cplx>(int, double, double, int);

}  // namespace ssg
