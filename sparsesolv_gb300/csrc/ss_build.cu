// ss_build.cu -- CSR from COO triplets on the device.
//
// The reference assembles a matrix on the host: SparseBuilder accumulates
// entries with += into one std::map per row (include/SparseSolv/SparseBuilder.hpp:53-80,
// src/SparseBuilder.cpp:107-141), or the COO constructor hands triplets to
// Eigen's setFromTriplets (src/SparseMat.cpp:80-104). Either way the result is
// CSR with ascending columns, an entry that occurs several times being summed
// one value after another in input order. Here: an LSD radix sort of the
// entries keyed on row * n + col, stable in every pass (so equal keys keep
// their input order), then one thread per run of equal keys sums its values
// in that order, and a scan of the per-row counts gives the row pointers.
#include "sparsesolv_gb300.h"
#include "ss_internal.cuh"
#include "ss_solver.cuh"

namespace ssg {

constexpr int RX_BITS = 8;
constexpr int RX_BUCKETS = 1 << RX_BITS;
constexpr int RX_CHUNK = 2048;  // entries a warp ranks in one pass

__global__ void k_coo_keys(int m, const int *rows, const int *cols, int n, unsigned long long *key, int *idx,
                           int *bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int r = rows[i], c = cols[i];
    if (r < 0 || r >= n || c < 0 || c >= n) {
        atomicExch(bad, 1);
        r = 0;
        c = 0;
    }
    key[i] = (unsigned long long)r * (unsigned long long)n + (unsigned long long)c;
    idx[i] = i;
}

// digit histogram per chunk of entries: cnt[digit * nchunks + chunk]; one warp per chunk
__global__ void k_digit_hist(int m, const unsigned long long *key, int shift, int nchunks, int *cnt) {
    const int lane = threadIdx.x & 31;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= nchunks) return;
    const int a = c * RX_CHUNK, b = min(m, a + RX_CHUNK);
    for (int base = a; base < b; base += 32) {
        const int i = base + lane;
        const int d = i < b ? (int)((key[i] >> shift) & (RX_BUCKETS - 1)) : -1;
        const unsigned mm = __match_any_sync(0xffffffffu, d);
        if (i < b && lane == __ffs(mm) - 1) cnt[(size_t)d * nchunks + c] += __popc(mm);
        __syncwarp();
    }
}

// stable scatter by digit: within a chunk, entries keep their order
__global__ void k_digit_scatter(int m, const unsigned long long *kin, const int *iin, int shift, int nchunks, int *off,
                                unsigned long long *kout, int *iout) {
    const int lane = threadIdx.x & 31;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= nchunks) return;
    const int a = c * RX_CHUNK, b = min(m, a + RX_CHUNK);
    const unsigned lt = (1u << lane) - 1u;
    for (int base = a; base < b; base += 32) {
        const int i = base + lane;
        const unsigned long long k = i < b ? kin[i] : 0ull;
        const int d = i < b ? (int)((k >> shift) & (RX_BUCKETS - 1)) : -1;
        const unsigned mm = __match_any_sync(0xffffffffu, d);
        int o = 0;
        if (i < b) o = off[(size_t)d * nchunks + c];
        __syncwarp();
        if (i < b) {
            const int pos = o + __popc(mm & lt);
            kout[pos] = k;
            iout[pos] = iin[i];
            if (lane == __ffs(mm) - 1) off[(size_t)d * nchunks + c] = o + __popc(mm);
        }
        __syncwarp();
    }
}

__global__ void k_run_heads(int m, const unsigned long long *key, int *head) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) head[i] = (i == 0 || key[i] != key[i - 1]) ? 1 : 0;
}

// one thread per run of equal keys: its values summed in input order
template <typename T>
__global__ void k_sum_runs(int m, const unsigned long long *key, const int *idx, const int *pos, const T *vin, int n,
                           int *ci, T *vout, int *rowcnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || !(i == 0 || key[i] != key[i - 1])) return;
    const unsigned long long k = key[i];
    T acc = vin[idx[i]];
    for (int j = i + 1; j < m && key[j] == k; ++j) acc = acc + vin[idx[j]];
    const int p = pos[i];
    const int r = (int)(k / (unsigned long long)n);
    ci[p] = (int)(k % (unsigned long long)n);
    vout[p] = acc;
    atomicAdd(rowcnt + r, 1);
}

template <typename T>
static void coo_to_csr(int n, int m, const int *rows, const int *cols, const T *vals, DBuf &rp, DBuf &ci, DBuf &val,
                       int &nnz_out, cudaStream_t s) {
    DBuf key0, key1, idx0, idx1, head, small, tmp;
    key0.alloc(sizeof(unsigned long long) * (size_t)m);
    key1.alloc(sizeof(unsigned long long) * (size_t)m);
    idx0.alloc(sizeof(int) * (size_t)m);
    idx1.alloc(sizeof(int) * (size_t)m);
    small.alloc(4 * sizeof(int));
    SSG_CUDA(cudaMemsetAsync(small.p, 0, 4 * sizeof(int), s));
    int *bad = small.as<int>(), *total = small.as<int>() + 1;
    k_coo_keys<<<div_up(m, 256), 256, 0, s>>>(m, rows, cols, n, key0.as<unsigned long long>(), idx0.as<int>(), bad);
    SSG_LAUNCHED();
    // key bits: row * n + col < n^2
    const unsigned long long kmax = (unsigned long long)n * (unsigned long long)n - 1ull;
    int bits = 0;
    while (bits < 64 && (kmax >> bits) != 0ull) ++bits;
    const int nchunks = div_up(m, RX_CHUNK);
    DBuf cnt;
    cnt.alloc(sizeof(int) * ((size_t)RX_BUCKETS * nchunks + 1));
    for (int shift = 0; shift < bits; shift += RX_BITS) {
        SSG_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * ((size_t)RX_BUCKETS * nchunks + 1), s));
        k_digit_hist<<<div_up(nchunks * 32, 256), 256, 0, s>>>(m, key0.as<unsigned long long>(), shift, nchunks,
                                                               cnt.as<int>());
        SSG_LAUNCHED();
        scan_exclusive(cnt.as<int>(), RX_BUCKETS * nchunks, nullptr, s, tmp);
        k_digit_scatter<<<div_up(nchunks * 32, 256), 256, 0, s>>>(m, key0.as<unsigned long long>(), idx0.as<int>(),
                                                                  shift, nchunks, cnt.as<int>(),
                                                                  key1.as<unsigned long long>(), idx1.as<int>());
        SSG_LAUNCHED();
        std::swap(key0, key1);
        std::swap(idx0, idx1);
    }
    head.alloc(sizeof(int) * ((size_t)m + 1));
    k_run_heads<<<div_up(m, 256), 256, 0, s>>>(m, key0.as<unsigned long long>(), head.as<int>());
    SSG_LAUNCHED();
    scan_exclusive(head.as<int>(), m, total, s, tmp);
    int hv[2] = {0, 0};
    SSG_CUDA(cudaMemcpyAsync(hv, small.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaStreamSynchronize(s));
    if (hv[0]) throw Error{SSG_ERR_ARG, "a COO entry lies outside [0, n) x [0, n)"};
    nnz_out = hv[1];
    rp.ensure(sizeof(int) * ((size_t)n + 1));
    ci.ensure(sizeof(int) * ((size_t)nnz_out + 1));
    val.ensure(sizeof(T) * ((size_t)nnz_out + 1));
    SSG_CUDA(cudaMemsetAsync(rp.p, 0, sizeof(int) * ((size_t)n + 1), s));
    k_sum_runs<T><<<div_up(m, 256), 256, 0, s>>>(m, key0.as<unsigned long long>(), idx0.as<int>(), head.as<int>(),
                                                 vals, n, ci.as<int>(), val.as<T>(), rp.as<int>());
    SSG_LAUNCHED();
    scan_exclusive(rp.as<int>(), n + 1, nullptr, s, tmp);
    SSG_CUDA(cudaStreamSynchronize(s));
}

void Handle::set_matrix_coo(int n_, int m, const int *rows, const int *cols, const double *vals, int vt,
                            cudaMemcpyKind kind) {
    if (n_ <= 0 || m < 0 || (vt != SSG_REAL && vt != SSG_COMPLEX)) throw Error{SSG_ERR_ARG, "bad matrix arguments"};
    if ((unsigned long long)n_ * (unsigned long long)n_ >= (1ull << 62)) throw Error{SSG_ERR_ARG, "n too large"};
    const size_t vb = vt == SSG_COMPLEX ? 16 : 8;
    DBuf hr, hc, hv;
    const int *dr = rows, *dc = cols;
    const void *dv = vals;
    if (kind == cudaMemcpyHostToDevice && m > 0) {
        hr.alloc(sizeof(int) * (size_t)m);
        hc.alloc(sizeof(int) * (size_t)m);
        hv.alloc(vb * (size_t)m);
        SSG_CUDA(cudaMemcpyAsync(hr.p, rows, sizeof(int) * (size_t)m, cudaMemcpyHostToDevice, stream));
        SSG_CUDA(cudaMemcpyAsync(hc.p, cols, sizeof(int) * (size_t)m, cudaMemcpyHostToDevice, stream));
        SSG_CUDA(cudaMemcpyAsync(hv.p, vals, vb * (size_t)m, cudaMemcpyHostToDevice, stream));
        dr = hr.as<int>();
        dc = hc.as<int>();
        dv = hv.p;
    }
    int nz = 0;
    if (m == 0) {
        A_rp.ensure(sizeof(int) * ((size_t)n_ + 1));
        A_ci.ensure(sizeof(int));
        A_val.ensure(vb);
        SSG_CUDA(cudaMemsetAsync(A_rp.p, 0, sizeof(int) * ((size_t)n_ + 1), stream));
        SSG_CUDA(cudaStreamSynchronize(stream));
    } else if (vt == SSG_COMPLEX) {
        coo_to_csr<cplx>(n_, m, dr, dc, (const cplx *)dv, A_rp, A_ci, A_val, nz, stream);
    } else {
        coo_to_csr<double>(n_, m, dr, dc, (const double *)dv, A_rp, A_ci, A_val, nz, stream);
    }
    n = n_;
    nnz = nz;
    vtype = vt;
    ++version;
    ++pattern_id;
    pat_version = ~0ull;
    ltb_ready = ub_ready = false;
    fac_valid = sgs_valid = dad_valid = false;
    note_row_lengths(nullptr);
}

}  // namespace ssg
