// ss_internal.cuh -- host-side internal interfaces between the translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "ss_common.cuh"
#include "ss_push_plan.hpp"

namespace ssg {

// Thrown inside the library, converted to a return code at the C ABI.
struct Error {
    int code;
    std::string msg;
};

void cuda_check(cudaError_t e, const char *what);
#define SSG_CUDA(call) ::ssg::cuda_check((call), #call)
// after every kernel launch: count it and surface launch errors
void note_launch();
long long launch_count();
void add_launches(long long k);  // kernels run from a replayed graph (negative: captured, not run)
#define SSG_LAUNCHED() ::ssg::note_launch()

// ---------------------------------------------------------------- device memory
// Stream that device buffers are allocated and freed on (thread-local; set by
// the C ABI entry points to the handle's stream). A plain cudaFree waits for
// the whole device, so every handle or batch that frees a temporary would stall
// the work of all others; stream-ordered allocation (cudaMallocAsync /
// cudaFreeAsync on the owning stream) frees in order with that stream only.
// Null: synchronous cudaMalloc / cudaFree.
cudaStream_t &alloc_stream();
struct AllocStream {
    cudaStream_t prev;
    explicit AllocStream(cudaStream_t s) : prev(alloc_stream()) { alloc_stream() = s; }
    ~AllocStream() { alloc_stream() = prev; }
};

// Owning device buffer; freed on the stream it was allocated on, which
// therefore must outlive it (Handle keeps its stream in its first member).
struct DBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaStream_t s = nullptr;  // allocation stream (null: synchronous)
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    DBuf(DBuf &&o) noexcept : p(o.p), bytes(o.bytes), s(o.s) { o.p = nullptr; o.bytes = 0; o.s = nullptr; }
    DBuf &operator=(DBuf &&o) noexcept {
        if (this != &o) { release(); p = o.p; bytes = o.bytes; s = o.s; o.p = nullptr; o.bytes = 0; o.s = nullptr; }
        return *this;
    }
    ~DBuf() { release(); }
    void release();
    void alloc(size_t b);           // exact size, content undefined
    void ensure(size_t b);          // grow when smaller
    template <typename U>
    U *as() const { return (U *)p; }
};

// ---------------------------------------------------------------- push sweep plan (ss_push.cu)
// One-cluster push schedule of a level-ordered triangle (ss_push_plan.hpp): every
// CTA owns a contiguous chunk of each level, sums each row's entries oldest
// dependency first, and pushes each finished value into the shared memory of the
// CTAs that read it, so no barrier spans the cluster per level.
struct PushPlan {
    bool ready = false;
    int fail = 0;                 // value sizes found infeasible (bit 0: 4 bytes, 1: 8, 2: 16)
    int elem = 0, C = 0, nent = 0, npush = 0;
    int n = -1, nnz = -1, nlev = -1;  // shape of the triangle the plan was made for
    PushLayout lay{};
    DBuf tab;                     // per (level, CTA) int4 {record offset / 16, record bytes / 16, bytes received, 0}
    DBuf rec;                     // the level records; values refilled per factor and per sweep
    DBuf vmap, dval, dlv, drhs, perm;  // where the factor's values, 1/diagonal or D, and the rhs go in rec
    DBuf dnew;                    // (entry, row) pairs of the newest entries, stored as -(value * lvec[row])
    int nnew = 0;
    const void *key_val = nullptr, *key_lv = nullptr;
    unsigned long long key_epoch = ~0ull;
};

// ---------------------------------------------------------------- level-scheduled triangle
// One triangular factor in the layout the sweeps stream: rows in level order
// (level, then row id), each row's entries contiguous and in the original
// column order, column indices kept as original row ids.
struct Tri {
    int n = 0, nnz = 0, nlev = 0;
    int nnz_pad = 16;            // every per-entry array of this triangle (pci, psrc, codes, values) has nnz + nnz_pad slots
    bool lower = true;           // lower: deps j < i, diagonal last; upper: deps j > i, diagonal first
    DBuf level, perm, ipos;      // level[i], perm[t] = row, ipos[row] = t
    DBuf prp, pci, psrc;         // level-ordered CSR; psrc[k] = source value index
    std::vector<int> lptr;       // host copy of level pointers
    DBuf lptr_d;
    // cluster sweep plan (ss_cluster.cu)
    bool cl_ready = false;
    bool cl_p2p = false;         // neighbour-synchronised plan (IC sweeps only)
    int cl_fail = 0;             // plans found infeasible for this pattern: bit 0 lockstep, bit 1 neighbour-synchronised
    int cl_C = 0, cl_S = 0, cl_elem = 0, cl_ring_bytes = 0, cl_cap_r = 0, cl_cap_e = 0;
    DBuf cl_code;                // per level-ordered entry: row id, or -1 - (owner << 20 | ring slot)
    DBuf cl_tab;                 // per (level, CTA): rows [rs, re) and entries [e0, e1) of the chunk
    PushPlan push[3];            // push sweep plans (ss_push.cu), one per value size: 4, 8, 16 bytes
};

// ss_levels.cu
void scan_exclusive(int *d_in_out, int count, int *d_total, cudaStream_t s, DBuf &tmp);
// triangle of a CSR pattern (explicit zeros kept): rp/ci natural order -> trp/tci/tsrc
void triangle_pattern(int n, const int *rp, const int *ci, bool lower, DBuf &trp, DBuf &tci, DBuf &tsrc,
                      int &tnnz, cudaStream_t s, DBuf &tmp);
// transpose of a CSR pattern with sorted rows, tsrc[k] = entry of the source
void transpose_pattern(int n, int nnz, const int *rp, const int *ci, DBuf &trp, DBuf &tci, DBuf &tsrc,
                       cudaStream_t s, DBuf &tmp);
// level schedule + level-ordered copy of a triangle given in natural order;
// src (may be null) is composed into psrc.
void build_tri(Tri &T, int n, int nnz, const int *rp, const int *ci, const int *src, bool lower,
               int *d_err, cudaStream_t s, DBuf &tmp);
// out[k] = in[src[k]] for k < count (values of width sizeof(T))
template <typename T>
void gather_values(const int *src, const T *in, T *out, int count, cudaStream_t s);

// ss_factor.cu
// per entry of L: (start, length) of its dependency row in level order; longest row
void factor_plan(const Tri &L, DBuf &dep, int &max_row, cudaStream_t s);
// asynchronous; done[n] is scratch the caller owns
template <typename T>
void ic_factor(const Tri &L, T *lval, T *D, double alpha, int *d_err, int *d_ticket, cudaStream_t s,
               const int2 *dep, int max_row, int *done, int backoff_ns, const int *sub = nullptr, int nsub = 0);
// copy the factor rows of rows with a source row (rep_src[i] >= 0) from that row
template <typename T>
void copy_replica_rows(const Tri &L, const int *rep_src, T *lval, T *D, cudaStream_t s);
// level-ordered positions of the rows without a source row, ascending, into sub; returns their count
int own_rows(const Tri &L, const int *rep_src, DBuf &sub, cudaStream_t s);
// natural-order factor with library-owned scratch; returns an SSG_* code
int ic_factor_noalloc(int n, int nnz, const int *lrp, const int *lci, const void *val, void *lval, void *D,
                      double alpha, int vtype, cudaStream_t s);
template <typename T>
void diag_scaling(int n, const int *rp, const int *ci, const T *val, const T *b, T *d, T *bs, cudaStream_t s);
template <typename T>
void dad_values(int n, const int *rp, const int *ci, const T *val, const T *d, T *out, cudaStream_t s);
template <typename T>
void all_pivots_positive(int n, const T *D, int *d_flag, cudaStream_t s);

// ss_trsv.cu
enum SweepMode : int {
    SW_FWD_DIV = 0,   // out_i = (rhs_i - sum_{j<i} v_ij out_j) / v_ii        (diag last)
    SW_BWD_IC = 1,    // out_i = D_i * (-sum_{j>i} v_ij out_j) + aux_i         (diag first, skipped)
    SW_BWD_DIV = 2,   // out_i = (rhs_i - sum_{j>i} v_ij out_j) / v_ii        (diag first)
    SW_FWD_EIS = 3,   // y_i = (rhs_i - aux_i - sum v_ij y_j) / v_ii, out2_i = y_i + aux_i
};
template <typename T>
void sweep(const Tri &tri, const T *val, int mode, const T *rhs, const T *aux, const T *D, T *out, T *out2,
           int *d_ticket, int *d_err, cudaStream_t s);
// launch shape of the sweeps (tunable; 0 = automatic)
struct SweepCfg {
    int cta_per_sm = 0;   // resident CTAs per SM claiming rows (0: from the mean level width)
    int group = 0;        // lanes per row: 4, 8, 16 or 32 (0: from the mean row length)
    int backoff_ns = 0;   // __nanosleep between polls of an unsolved entry
    // batches: rows whose instance has ended are skipped (row -> instance, and the
    // instances' active flags act[instance * act_stride]); null for one system
    const int *row_inst = nullptr;
    const int *act = nullptr;
    int act_stride = 0;
};
template <typename T>
void inv_diag(const Tri &tri, const T *val, T *inv, cudaStream_t s);
int sweep_group(const Tri &tri);  // lanes per row from the mean row length

// ss_cluster.cu: one-cluster level-synchronous sweeps
int cluster_size_available();  // 16, 8 or 0
// p2p: neighbour-synchronised plan (no cluster barrier per level; IC sweeps only)
void cluster_plan(Tri &T, size_t elem_bytes, int ring_bytes, cudaStream_t s, DBuf &tmp, bool p2p);
struct KState;
// lvec: per-row vector in this triangle's level order (1/diagonal, or D for SW_BWD_IC);
// err: the handle's error word (bounded waits of the neighbour-synchronised sweep)
template <typename T>
void sweep_cluster(const Tri &tri, const T *val, int mode, const T *rhs, const T *aux, const T *lvec, T *out, T *out2,
                   const KState *st, int group, int *err, cudaStream_t s);

// ss_push.cu: one-cluster push sweeps (IC pair: SW_FWD_DIV with lvec = 1/diagonal, SW_BWD_IC with lvec = D)
// plan once per pattern and value size; false when a schedule does not fit (then another sweep serves);
// the count triangles of one call are planned side by side on host threads
bool push_plan(Tri *const *tris, int count, size_t elem_bytes, cudaStream_t s);
// val: the triangle's values in its level-ordered layout, lvec: per level-ordered row; epoch changes whenever
// the values behind val / lvec change (the records are refilled then)
template <typename T>
void sweep_push(Tri &tri, const T *val, int mode, const T *rhs, const T *lvec, unsigned long long epoch, T *out,
                const KState *st, int *err, cudaStream_t s);

// ss_spmv_vec.cu -- see the Krylov state there
struct KState;
template <typename T>
void spmv(int n, int group, const int *rp, const int *ci, const T *val, const T *x, T *y, cudaStream_t s);
size_t part_bytes();
// nat2lev[e] = level-ordered position of entry e of the natural-order triangle (rp)
void level_positions(const Tri &T, const int *rp, int *nat2lev, cudaStream_t s);

}  // namespace ssg
