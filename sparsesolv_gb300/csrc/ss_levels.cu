// ss_levels.cu -- integer work on the GPU: triangles, transposes, level sets,
// level permutation and level-ordered copies of the triangular factors.
//
// The reference sweeps rows strictly in natural order
// (MatSolverBase::IC_frbc_process, src/MatSolverBase.cpp:181-199); the level
// schedule computed here is the dependency structure of that order:
//   forward  level(i) = 1 + max{level(j) : j < i, L_ij stored}   (0 if none)
//   backward level(i) = 1 + max{level(j) : j > i, U_ij stored}   (0 if none)
// and the permutation lists rows by (level, row id). All of it is integer
// work and is bit-identical to the host recomputation in the oracle.
#include <atomic>

#include "ss_internal.cuh"

namespace ssg {

void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw Error{-2, std::string(what) + ": " + cudaGetErrorString(e)};
}

static std::atomic<long long> g_launches{0};
void note_launch() {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cuda_check(cudaGetLastError(), "kernel launch");
}
long long launch_count() { return g_launches.load(); }
void add_launches(long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

cudaStream_t &alloc_stream() {
    static thread_local cudaStream_t s = nullptr;
    return s;
}

void DBuf::release() {
    if (p) {
        if (s)
            cudaFreeAsync(p, s);
        else
            cudaFree(p);
    }
    p = nullptr;
    bytes = 0;
    s = nullptr;
}
void DBuf::alloc(size_t b) {
    release();
    if (b == 0) b = 16;
    s = alloc_stream();
    cudaError_t e = s ? cudaMallocAsync(&p, b, s) : cudaMalloc(&p, b);
    if (e != cudaSuccess) {
        p = nullptr;
        (void)cudaGetLastError();
        throw Error{-5, "cudaMalloc of " + std::to_string(b) + " bytes failed"};
    }
    bytes = b;
}
void DBuf::ensure(size_t b) {
    if (bytes < b || !p) alloc(b);
}

// ---------------------------------------------------------------- exclusive scan
constexpr int SCAN_T = 512;
constexpr int SCAN_PER = 4;
constexpr int SCAN_TILE = SCAN_T * SCAN_PER;

__global__ void k_scan_tile(int *data, int count, int *sums) {
    __shared__ int warp_tot[SCAN_T / 32];
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER;
    int v[SCAN_PER];
    int local = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) {
        v[k] = (base + k < count) ? data[base + k] : 0;
        local += v[k];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = local;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += t;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int w = (lane < SCAN_T / 32) ? warp_tot[lane] : 0;
        int wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += t;
        }
        if (lane < SCAN_T / 32) warp_tot[lane] = wi - w;  // exclusive warp offsets
        if (lane == SCAN_T / 32 - 1 && sums) sums[blockIdx.x] = wi;
    }
    __syncthreads();
    int run = warp_tot[wid] + incl - local;
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) {
        if (base + k < count) data[base + k] = run;
        run += v[k];
    }
}

__global__ void k_scan_add(int *data, int count, const int *sums) {
    const int i = blockIdx.x * SCAN_TILE + threadIdx.x;
    const int add = sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) {
        const int j = i + k * SCAN_T;
        if (j < count) data[j] += add;
    }
}

__global__ void k_scan_total(const int *data, const int *last_in, int count, int *total) {
    // total = exclusive[count-1] + original last value
    *total = data[count - 1] + *last_in;
}

static void scan_rec(int *d, int count, cudaStream_t s, std::vector<DBuf> &pool, size_t depth) {
    const int nb = div_up(count, SCAN_TILE);
    if (pool.size() <= depth) pool.emplace_back();
    pool[depth].ensure(sizeof(int) * (size_t)(nb + 1));
    int *sums = pool[depth].as<int>();
    k_scan_tile<<<nb, SCAN_T, 0, s>>>(d, count, sums);
    SSG_LAUNCHED();
    if (nb > 1) {
        scan_rec(sums, nb, s, pool, depth + 1);
        k_scan_add<<<nb, SCAN_T, 0, s>>>(d, count, sums);
        SSG_LAUNCHED();
    }
}

void scan_exclusive(int *d, int count, int *d_total, cudaStream_t s, DBuf &tmp) {
    if (count <= 0) {
        if (d_total) SSG_CUDA(cudaMemsetAsync(d_total, 0, sizeof(int), s));
        return;
    }
    tmp.ensure(sizeof(int));
    if (d_total) SSG_CUDA(cudaMemcpyAsync(tmp.as<int>(), d + count - 1, sizeof(int), cudaMemcpyDeviceToDevice, s));
    std::vector<DBuf> pool;
    scan_rec(d, count, s, pool, 0);
    if (d_total) {
        k_scan_total<<<1, 1, 0, s>>>(d, tmp.as<int>(), count, d_total);
        SSG_LAUNCHED();
    }
    SSG_CUDA(cudaStreamSynchronize(s));  // pool buffers are released on return
}

// ---------------------------------------------------------------- triangles
__global__ void k_tri_count(int n, const int *rp, const int *ci, int lower, int *cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    if (i == n) { cnt[n] = 0; return; }
    int c = 0;
    for (int k = rp[i]; k < rp[i + 1]; ++k) c += lower ? (ci[k] <= i) : (ci[k] >= i);
    cnt[i] = c;
}

__global__ void k_tri_fill(int n, const int *rp, const int *ci, int lower, const int *trp, int *tci, int *tsrc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int o = trp[i];
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
        const int c = ci[k];
        if (lower ? (c <= i) : (c >= i)) {
            tci[o] = c;
            tsrc[o] = k;
            ++o;
        }
    }
}

void triangle_pattern(int n, const int *rp, const int *ci, bool lower, DBuf &trp, DBuf &tci, DBuf &tsrc,
                      int &tnnz, cudaStream_t s, DBuf &tmp) {
    trp.ensure(sizeof(int) * (size_t)(n + 1));
    k_tri_count<<<div_up(n + 1, 256), 256, 0, s>>>(n, rp, ci, lower ? 1 : 0, trp.as<int>());
    SSG_LAUNCHED();
    scan_exclusive(trp.as<int>(), n + 1, nullptr, s, tmp);
    int h = 0;
    SSG_CUDA(cudaMemcpyAsync(&h, trp.as<int>() + n, sizeof(int), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaStreamSynchronize(s));
    tnnz = h;
    tci.ensure(sizeof(int) * (size_t)(h + 1));
    tsrc.ensure(sizeof(int) * (size_t)(h + 1));
    if (n == 0) return;
    k_tri_fill<<<div_up(n, 256), 256, 0, s>>>(n, rp, ci, lower ? 1 : 0, trp.as<int>(), tci.as<int>(), tsrc.as<int>());
    SSG_LAUNCHED();
}

// ---------------------------------------------------------------- transpose
__global__ void k_col_count(int nnz, const int *ci, int *cnt) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) atomicAdd(&cnt[ci[k]], 1);
}

__global__ void k_transpose_fill(int n, const int *rp, const int *ci, int *fill, int *tci, int *tsrc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
        const int pos = atomicAdd(&fill[ci[k]], 1);
        tci[pos] = i;
        tsrc[pos] = k;
    }
}

// rows of a transpose arrive in arbitrary order; sorting by column makes the
// result deterministic (columns within a row are distinct)
__global__ void k_sort_segments(int n, const int *rp, int *ci, int *src) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int a = rp[i], b = rp[i + 1];
    for (int k = a + 1; k < b; ++k) {
        const int c = ci[k], s = src[k];
        int j = k - 1;
        while (j >= a && ci[j] > c) {
            ci[j + 1] = ci[j];
            src[j + 1] = src[j];
            --j;
        }
        ci[j + 1] = c;
        src[j + 1] = s;
    }
}

void transpose_pattern(int n, int nnz, const int *rp, const int *ci, DBuf &trp, DBuf &tci, DBuf &tsrc,
                       cudaStream_t s, DBuf &tmp) {
    trp.ensure(sizeof(int) * (size_t)(n + 1));
    tci.ensure(sizeof(int) * (size_t)(nnz + 1));
    tsrc.ensure(sizeof(int) * (size_t)(nnz + 1));
    SSG_CUDA(cudaMemsetAsync(trp.p, 0, sizeof(int) * (size_t)(n + 1), s));
    if (n == 0 || nnz == 0) {
        SSG_CUDA(cudaStreamSynchronize(s));
        return;
    }
    k_col_count<<<div_up(nnz, 256), 256, 0, s>>>(nnz, ci, trp.as<int>());
    SSG_LAUNCHED();
    scan_exclusive(trp.as<int>(), n + 1, nullptr, s, tmp);
    DBuf fill;
    fill.alloc(sizeof(int) * (size_t)(n + 1));
    SSG_CUDA(cudaMemcpyAsync(fill.p, trp.p, sizeof(int) * (size_t)(n + 1), cudaMemcpyDeviceToDevice, s));
    k_transpose_fill<<<div_up(n, 256), 256, 0, s>>>(n, rp, ci, fill.as<int>(), tci.as<int>(), tsrc.as<int>());
    SSG_LAUNCHED();
    k_sort_segments<<<div_up(n, 256), 256, 0, s>>>(n, trp.as<int>(), tci.as<int>(), tsrc.as<int>());
    SSG_LAUNCHED();
    SSG_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------- level sets
// A group of LV_G lanes per row; a CTA claims LV_ROWS consecutive rows per
// ticket, in dependency order (increasing row id for the forward triangle,
// decreasing for the backward one), so every row a group waits on was claimed
// earlier by a running group and the waits always end. Groups of one warp
// reduce with group-local masks (one may wait on another). Each wait is also
// bounded in time.
constexpr int LV_G = 8;
constexpr int LV_THREADS = 128;
constexpr int LV_ROWS = LV_THREADS / LV_G;

__global__ void __launch_bounds__(LV_THREADS) k_levels(int n, const int *rp, const int *ci, int lower, int *level,
                                                       int *ticket, int *nlev, int *err) {
    __shared__ int s_base;
    const int g = threadIdx.x / LV_G, gl = threadIdx.x % LV_G;
    const unsigned gm = group_mask(LV_G);
    int my_max = 0;
    for (;;) {
        if (threadIdx.x == 0) s_base = atomicAdd(ticket, LV_ROWS);
        __syncthreads();
        const int base = s_base;
        __syncthreads();
        if (base >= n) break;
        const int t = base + g;
        if (t < n) {
            const int row = lower ? t : n - 1 - t;
            int l = 0;
            for (int k = rp[row] + gl; k < rp[row + 1]; k += LV_G) {
                const int c = ci[k];
                if (lower ? (c < row) : (c > row)) {
                    const volatile int *pl = level + c;
                    int v = *pl;
                    if (v < 0) {
                        const unsigned long long start = gtimer();
                        int polls = 0;
                        while ((v = *pl) < 0) {
                            __nanosleep(32);
                            if ((++polls & 63) == 0) {
                                if (*(volatile int *)err) { v = 0; break; }
                                if (gtimer() - start > spin_limit_ns(err)) {
                                    atomicExch(err, ERR_TIMEOUT);
                                    v = 0;
                                    break;
                                }
                            }
                        }
                    }
                    l = max(l, v + 1);
                }
            }
#pragma unroll
            for (int m = LV_G / 2; m >= 1; m >>= 1) l = max(l, __shfl_xor_sync(gm, l, m));
            if (gl == 0) *(volatile int *)(level + row) = l;
            my_max = max(my_max, l);
        }
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) my_max = max(my_max, __shfl_xor_sync(0xffffffffu, my_max, m));
    if ((threadIdx.x & 31) == 0) atomicMax(nlev, my_max + 1);
}

// histogram of levels per chunk of rows: cnt[l * nchunks + c]; one warp per chunk
__global__ void k_level_hist(int n, const int *level, int chunk, int nchunks, int *cnt) {
    const int lane = threadIdx.x & 31;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= nchunks) return;
    const int a = c * chunk, b = min(n, a + chunk);
    for (int base = a; base < b; base += 32) {
        const int row = base + lane;
        const int lv = row < b ? level[row] : -1;
        const unsigned m = __match_any_sync(0xffffffffu, lv);
        if (row < b && lane == __ffs(m) - 1) cnt[(size_t)lv * nchunks + c] += __popc(m);
        __syncwarp();
    }
}

// stable scatter of rows into level order
__global__ void k_level_scatter(int n, const int *level, int chunk, int nchunks, int *off, int *perm, int *ipos) {
    const int lane = threadIdx.x & 31;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= nchunks) return;
    const int a = c * chunk, b = min(n, a + chunk);
    const unsigned lt = (1u << lane) - 1u;
    for (int base = a; base < b; base += 32) {
        const int row = base + lane;
        const int lv = row < b ? level[row] : -1;
        const unsigned m = __match_any_sync(0xffffffffu, lv);
        int o = 0;
        if (row < b) o = off[(size_t)lv * nchunks + c];
        __syncwarp();
        if (row < b) {
            const int pos = o + __popc(m & lt);
            perm[pos] = row;
            ipos[row] = pos;
            if (lane == __ffs(m) - 1) off[(size_t)lv * nchunks + c] = o + __popc(m);
        }
        __syncwarp();
    }
}

__global__ void k_extract_lptr(int nlev, int nchunks, const int *off, int n, int *lptr) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l < nlev) lptr[l] = off[(size_t)l * nchunks];
    if (l == nlev) lptr[nlev] = n;
}

__global__ void k_perm_len(int n, const int *perm, const int *trp, int *len) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > n) return;
    if (t == n) { len[n] = 0; return; }
    const int r = perm[t];
    len[t] = trp[r + 1] - trp[r];
}

__global__ void k_perm_copy(int n, const int *perm, const int *trp, const int *tci, const int *src, const int *prp,
                            int *pci, int *psrc) {
    const int lane = threadIdx.x & 31;
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (t >= n) return;
    const int r = perm[t];
    const int a = trp[r], len = trp[r + 1] - a, o = prp[t];
    for (int k = lane; k < len; k += 32) {
        pci[o + k] = tci[a + k];
        psrc[o + k] = src ? src[a + k] : a + k;
    }
}

void build_tri(Tri &T, int n, int nnz, const int *rp, const int *ci, const int *src, bool lower, int *d_err,
               cudaStream_t s, DBuf &tmp) {
    T.n = n;
    T.nnz = nnz;
    T.lower = lower;
    T.cl_ready = false;
    T.cl_fail = 0;
    T.cl_elem = 0;
    // a new pattern: the push plan (records, codes, slots) belongs to the old one
    for (PushPlan &P : T.push) {
        P.ready = false;
        P.fail = 0;
        P.elem = 0;
        P.n = P.nnz = P.nlev = -1;
        P.key_val = P.key_lv = nullptr;
        P.key_epoch = ~0ull;
    }
    T.level.ensure(sizeof(int) * (size_t)n);
    T.perm.ensure(sizeof(int) * (size_t)n);
    T.ipos.ensure(sizeof(int) * (size_t)n);
    DBuf small;
    small.alloc(2 * sizeof(int));
    int *ticket = small.as<int>(), *nlev_d = small.as<int>() + 1;
    SSG_CUDA(cudaMemsetAsync(small.p, 0, 2 * sizeof(int), s));
    SSG_CUDA(cudaMemsetAsync(T.level.p, 0xFF, sizeof(int) * (size_t)n, s));
    if (n > 0) {
        int dev = 0, sms = 0;
        SSG_CUDA(cudaGetDevice(&dev));
        SSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int blocks = min(div_up(n, LV_ROWS), sms * 2);
        k_levels<<<blocks, LV_THREADS, 0, s>>>(n, rp, ci, lower ? 1 : 0, T.level.as<int>(), ticket, nlev_d, d_err);
        SSG_LAUNCHED();
    }
    int hv[2] = {0, 0};
    SSG_CUDA(cudaMemcpyAsync(hv, small.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    int herr = 0;
    SSG_CUDA(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaStreamSynchronize(s));
    if (herr) throw Error{-4, "level schedule: a dependency wait timed out"};
    const int nlev = n > 0 ? hv[1] : 0;
    T.nlev = nlev;
    // chunked stable counting sort by level; the chunk grows with the level
    // count so that the (levels x chunks) table stays bounded
    long long chunk = 1024;
    const long long budget = 32ll << 20;
    while ((long long)nlev * div_up(n, (int)chunk) > budget) chunk *= 2;
    const int nchunks = max(1, div_up(n, (int)chunk));
    const size_t cells = (size_t)nlev * nchunks;
    DBuf cnt;
    cnt.alloc(sizeof(int) * (cells + 1));
    SSG_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * (cells + 1), s));
    if (n > 0) {
        k_level_hist<<<div_up((long long)nchunks * 32, 256), 256, 0, s>>>(n, T.level.as<int>(), (int)chunk, nchunks,
                                                                           cnt.as<int>());
        SSG_LAUNCHED();
        scan_exclusive(cnt.as<int>(), (int)cells, nullptr, s, tmp);
        T.lptr_d.ensure(sizeof(int) * (size_t)(nlev + 1));
        k_extract_lptr<<<div_up(nlev + 1, 256), 256, 0, s>>>(nlev, nchunks, cnt.as<int>(), n, T.lptr_d.as<int>());
        SSG_LAUNCHED();
        k_level_scatter<<<div_up((long long)nchunks * 32, 256), 256, 0, s>>>(n, T.level.as<int>(), (int)chunk, nchunks,
                                                                              cnt.as<int>(), T.perm.as<int>(),
                                                                              T.ipos.as<int>());
        SSG_LAUNCHED();
    } else {
        T.lptr_d.ensure(sizeof(int));
        SSG_CUDA(cudaMemsetAsync(T.lptr_d.p, 0, sizeof(int), s));
    }
    T.lptr.assign(nlev + 1, 0);
    SSG_CUDA(cudaMemcpyAsync(T.lptr.data(), T.lptr_d.p, sizeof(int) * (size_t)(nlev + 1), cudaMemcpyDeviceToHost, s));
    // level-ordered copy of the rows
    T.prp.ensure(sizeof(int) * (size_t)(n + 1));
    T.pci.ensure(sizeof(int) * (size_t)(nnz + T.nnz_pad));
    T.psrc.ensure(sizeof(int) * (size_t)(nnz + T.nnz_pad));
    SSG_CUDA(cudaMemsetAsync(T.pci.p, 0, sizeof(int) * (size_t)(nnz + T.nnz_pad), s));
    k_perm_len<<<div_up(n + 1, 256), 256, 0, s>>>(n, T.perm.as<int>(), rp, T.prp.as<int>());
    SSG_LAUNCHED();
    scan_exclusive(T.prp.as<int>(), n + 1, nullptr, s, tmp);
    if (n > 0) {
        k_perm_copy<<<div_up((long long)n * 32, 256), 256, 0, s>>>(n, T.perm.as<int>(), rp, ci, src, T.prp.as<int>(),
                                                                    T.pci.as<int>(), T.psrc.as<int>());
        SSG_LAUNCHED();
    }
    SSG_CUDA(cudaStreamSynchronize(s));
}

__global__ void k_level_positions(int n, const int *rp, const int *ipos, const int *prp, int *nat2lev) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int base = prp[ipos[i]];
    for (int k = rp[i]; k < rp[i + 1]; ++k) nat2lev[k] = base + (k - rp[i]);
}

void level_positions(const Tri &T, const int *rp, int *nat2lev, cudaStream_t s) {
    if (T.n == 0) return;
    k_level_positions<<<div_up(T.n, 256), 256, 0, s>>>(T.n, rp, T.ipos.as<int>(), T.prp.as<int>(), nat2lev);
    SSG_LAUNCHED();
}

template <typename T>
__global__ void k_gather(const int *src, const T *in, T *out, int count) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < count) out[k] = in[src[k]];
}

template <typename T>
void gather_values(const int *src, const T *in, T *out, int count, cudaStream_t s) {
    if (count <= 0) return;
    k_gather<T><<<div_up(count, 256), 256, 0, s>>>(src, in, out, count);
    SSG_LAUNCHED();
}
template void gather_values<int>(const int *, const int *, int *, int, cudaStream_t);
template void gather_values<double>(const int *, const double *, double *, int, cudaStream_t);
template void gather_values<cplx>(const int *, const cplx *, cplx *, int, cudaStream_t);
template void gather_values<float>(const int *, const float *, float *, int, cudaStream_t);
template void gather_values<cplxf>(const int *, const cplxf *, cplxf *, int, cudaStream_t);

}  // namespace ssg
