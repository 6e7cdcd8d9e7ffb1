// ss_solver.cuh -- the solver handle behind the C ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "sparsesolv_gb300.h"
#include "ss_internal.cuh"
#include "ss_krylov.cuh"

namespace ssg {

// per-kernel-class event timing (ssg_set_profiling)
enum : int { PC_FWD = 0, PC_BWD = 1, PC_SPMV = 2, PC_VEC = 3, PC_FACTOR = 4, PC_LEVELS = 5, PC_N = 6 };
struct ProfRec {
    int cls, iter;
    bool pre;  // launched before the iteration's convergence decision
    cudaEvent_t a, b;
    double bytes;
};
struct Prof {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<ProfRec> recs;
    double ms[PC_N] = {};
    long long launches[PC_N] = {};
    double bytes[PC_N] = {};
    int iter = 0;
    bool pre = true;
};

// Owns the handle's stream. First member of Handle, so it is destroyed last:
// the other members' device buffers are freed in order on this stream.
struct StreamGuard {
    cudaStream_t s = nullptr;
    ~StreamGuard() {
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
};

struct Handle {
    StreamGuard sg;
    int device = 0;
    cudaStream_t stream = nullptr;
    ssg_options opt{};
    std::string last_error;

    // ---- the matrix, natural order (SparseMat's CSR)
    int n = 0, nnz = 0, vtype = -1;
    uint64_t version = 0;     // bumps on every set_matrix and values update
    uint64_t pattern_id = 0;  // bumps when set_matrix brings a different sparsity pattern
    DBuf A_rp, A_ci, A_val;

    // ---- patterns and level schedules (depend on the sparsity pattern)
    uint64_t pat_version = ~0ull;
    DBuf Lnat_rp, Lnat_ci, Lnat_src;  // lower(A), src -> A entries
    int nnzL = 0;
    DBuf Unat_rp, Unat_ci, Unat_src;  // upper(A), src -> A entries
    int nnzU = 0;
    Tri Lf;          // forward schedule over lower(A); psrc -> A entries
    Tri Ltb;         // backward schedule over trans(lower(A)); psrc -> positions of Lf
    bool ltb_ready = false;
    Tri Ub;          // backward schedule over upper(A); psrc -> A entries
    bool ub_ready = false;
    DBuf nat2lev;    // natural lower entry -> position in Lf
    DBuf dep;        // per entry of Lf: (start, length) of its dependency row
    int max_row = 0; // longest row of Lf
    DBuf done_buf;   // factor row flags

    // ---- values
    DBuf Lval, Ltval, Cval, Uval, Dvec;  // factor (Lf / Ltb layouts), SGS triangles, 1/pivot
    DBuf invL, invC, invU;               // reciprocal diagonals (natural order) for the dividing sweeps
    DBuf invL_lev, D_lev, invC_lev, invU_lev;  // the same in the level order of the sweep that reads them
    bool fac_valid = false;
    uint64_t fac_version = 0;
    double fac_alpha_req = 0.0, alpha_used = 0.0;
    int fac_scaled = -1;
    bool sgs_valid = false;
    uint64_t sgs_version = 0;
    DBuf dscale, dad;  // diagonal scaling d and D A D values
    bool dad_valid = false;
    uint64_t dad_version = 0;

    // ---- work space
    DBuf vec[12];
    DBuf part, state, logbuf, small;  // small: ticket[4], err[1], pad, doubles[8]
    KState *h_state = nullptr;        // pinned
    double *h_scal = nullptr;         // pinned scratch

    // ---- results of the last solve
    std::vector<double> residual_log;
    int iters = 0;
    double t_setup_ms = 0.0, t_iter_ms = 0.0;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};

    // launch tuning (ssg_set_tuning)
    SweepCfg swcfg;
    int fac_backoff_ns = 0;
    bool use_inv_diag = true;
    int sweep_mode = 0;            // 0 auto (default), 1 sync-free, 2 cluster, 3 neighbour-synchronised cluster,
                                   // 4 push (one cluster, no cluster-wide barrier; IC pair)
    unsigned long long fac_epoch = 0;  // bumped whenever the factor values change (push records refill)
    int batch_group = 0;           // lanes a row in the sweeps of the owning C handle's internal batch (0: auto)
    int spmv_group_req = 0;        // lanes a row in the SpMV (0: from the row-length distribution)
    double spmv_len = 0.0;         // nonzero-weighted median row length of the current pattern
    int spmv_lanes() const { return spmv_group_req ? spmv_group_req : spmv_group(spmv_len, vtype == SSG_COMPLEX); }
    void note_row_lengths(const int *host_rp);  // the pattern changed: its row-length distribution (host or device rp)
    // rows whose factor is a copy of another row's (a batch holds a system once per
    // right-hand side): only the rows without a source are factored
    DBuf rep_src;                  // [n] source row or -1
    bool rep_on = false;
    DBuf fac_sub;                  // level-ordered positions of the rows factored
    int fac_sub_n = 0;
    bool fac_sub_valid = false;
    void set_replicas(const std::vector<int> &src);  // empty: every row is factored
    int cl_ring_bytes = 16 * 1024; // distributed shared-memory ring per CTA
    int cl_ring_bytes_p2p = 24 * 1024;  // its ring in mode 3 (producers may run ahead)
    int cl_group = 4;              // lanes per row in the cluster sweep
    // ic: an IC sweep (the only kind the neighbour-synchronised plan serves)
    bool cluster_ok(Tri &t, size_t elem, bool ic);
    bool push_ok(size_t elem);  // both triangles of the IC pair
    // the automatic mode may take the push sweep (off in the standalone batches: their
    // instances' bits must not depend on which schedule a batch's size leads to, and the
    // lane-summed schedules give the same bits at the same lanes a row)
    bool push_auto = true;

    Prof prof;
    int prof_begin(int cls);
    void prof_end(int idx, double bytes);
    void prof_flush(int iters_done);
    template <typename F>
    void timed(int cls, double bytes, F &&fn) {
        const int idx = prof_begin(cls);
        fn();
        prof_end(idx, bytes);
    }

    int *ticket() { return small.as<int>(); }
    int *err() { return small.as<int>() + 4; }  // err()[1]: spin limit of the bounded waits (us, 0: 4 s)
    int spin_limit_us = 0;                      // SSG_TUNE_SPIN_LIMIT_US
    void set_spin_limit(int us);
    double *dscal() { return (double *)(small.as<char>() + 64); }
    KState *st() { return state.as<KState>(); }

    Handle(int dev);
    ~Handle();
    void set_matrix(int n_, int nnz_, const int32_t *rp, const int32_t *ci, const double *val, int vt,
                    cudaMemcpyKind kind);
    void update_values(const double *val, cudaMemcpyKind kind);
    // the matrix from COO triplets, built on the device (ss_build.cu)
    void set_matrix_coo(int n_, int m, const int *rows, const int *cols, const double *vals, int vt,
                        cudaMemcpyKind kind);
    void values_changed();  // A_val was rewritten in place: keep the pattern, drop the factors
    void ensure_patterns(bool need_ltb, bool need_ub);
    void check_err(const char *where);
    template <typename T>
    void ensure_scaled();
    template <typename T>
    void ensure_factor(double alpha, bool scaled);
    template <typename T>
    void ensure_sgs();
    template <typename T>
    int solve(int method, double conv, int max_ite, double normB, const T *d_b, T *d_x);
    template <typename T>
    void apply_precond(const T *d_r, T *d_z, const KState *st);
    void ensure_work(size_t elem_bytes);
    // schedule autotuner (ssg_autotune): times the preconditioner for each
    // candidate sweep schedule on the current matrix and keeps the fastest
    struct TuneChoice {
        int mode, group, cta_per_sm;
        double ms;
    };
    template <typename T>
    TuneChoice autotune(bool keep_group, bool with_push = true);
};

// flux density B = curl A per voxel element (ss_post.cu)
// ss_voxel.cu: the voxel edge-element system assembled on the device into the handle's matrix
void voxel_assemble_any(Handle &h, int nx, int ny, int nz, const int *ex, const int *ey, const int *ez, int nunk,
                        const double *Ke, const double *Me, const double *Ce, const double *nu, const double *sig,
                        double omega, const double *tz, int vt, void *b, bool on_device);
void flux_density_any(Handle &h, int nx, int ny, int nz, double hx, double hy, double hz, const int *ex,
                      const int *ey, const int *ez, int nunk, const void *A, int vt, void *B, bool on_device);

}  // namespace ssg
