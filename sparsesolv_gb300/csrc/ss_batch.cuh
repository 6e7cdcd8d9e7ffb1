// ss_batch.cuh -- many independent systems solved in shared launches.
//
// The systems of a batch (each system once per right-hand side: an
// "instance") are concatenated into one block-diagonal matrix held by an
// ordinary Handle, so the pattern analysis, the level schedules, the IC(0)
// factor, the triangular sweeps and the SpMV are the single-system ones: a
// level of the block-diagonal triangle is the union of the instances' levels,
// and no row reads another instance's rows. What is per instance is the
// Krylov state: every reduction is cut into tiles of at most BATCH_TILE rows
// that never straddle two instances, each tile's partial is a fixed-order
// block sum, and one block adds an instance's tiles in order and runs that
// instance's scalar recurrence and convergence test. An instance's numbers
// therefore do not depend on which other instances share the batch.
#pragma once

#include <vector>

#include "ss_solver.cuh"

namespace ssg {

constexpr int BATCH_TILE = 2048;  // rows per reduction tile
constexpr int BATCH_PARTS = 6;    // doubles per tile partial (three complex dots)

// device view of a batch, passed to the kernels by value
struct BDev {
    int S, NT;
    const int2 *tile;     // [NT] rows [x, y) of the tile
    const int *tile_sys;  // [NT] instance of the tile
    const int *sys_tile;  // [S + 1] first tile of each instance
    const int *sys_row;   // [S + 1] first row of each instance
    KState *st;           // [S] per-instance state
    const int *act;       // per-instance activity mask: act[s * act_stride] (the state the launch follows)
    int act_stride;
    KState *ctl;          // batch control: active while any instance is
    double *part;         // [NT * BATCH_PARTS]
    unsigned *counter;    // last-block ticket
    double *logs;         // [S * log_stride] residual logs
    int log_stride;
};

// mixed precision: per-instance state of the FP64 refinement around the FP32 inner solves
struct OState {
    int active, status;
    int outer_it;     // refinement steps done
    int inner_total;  // inner iterations over all steps
    double normB, norm, scale, pad;
};

struct BatchSystem {
    int n = 0, nnz = 0, nrhs = 1;
    std::vector<int> rp, ci;
    std::vector<double> val;  // interleaved re/im for complex
    std::vector<double> B;    // nrhs right-hand sides, each n values (interleaved for complex)
};

struct Batch {
    Handle h;
    int vtype = -1;
    std::vector<BatchSystem> sys;
    // instances
    std::vector<int> inst_sys, inst_rhs, inst_row;  // per instance; inst_row has S + 1 entries
    std::vector<long long> inst_entry;              // first entry of each instance in the block-diagonal matrix
    int S = 0, NT = 0;
    bool assembled = false;
    bool rhs_dirty = true;  // right-hand sides changed since the last upload
    DBuf d_tile, d_tile_sys, d_sys_tile, d_sys_row, d_st, d_part, d_logs, d_ctl_counter;
    DBuf d_row_inst;  // instance of every row (the sync-free sweeps skip ended instances)
    KState *h_st = nullptr;   // pinned copy of the instance states
    int h_cap = 0;            // instances the pinned copies hold
    KState *h_ctl = nullptr;  // pinned copy of the control state
    cudaEvent_t ev_chunk = nullptr;
    // the running solve
    int method = SSG_METHOD_ICCG;
    int max_ite = 0, queued = 0, chunk = 2, iter_no = 0;
    bool running = false, log_on = true;
    // mixed precision (SSG_PREC_MIXED): FP32 copies of A and of the factor, FP32 inner vectors
    int precision = SSG_PREC_FP64;
    double inner_tol = 0.0;  // inner solves reduce the scaled residual by this factor (0: 1e-4 real, 1e-2 complex)
    double eff_inner_tol() const { return inner_tol > 0.0 ? inner_tol : (vtype == SSG_COMPLEX ? 1.0e-2 : 1.0e-4); }
    DBuf d_ost, d_octl, A32, L32, Lt32, invL32, invL32_lev, D32, D32_lev, v32[11];
    unsigned long long mix_epoch = 0;  // bumped whenever the FP32 factor copies are rewritten
    OState *h_ost = nullptr;
    KState *h_octl = nullptr;
    KState *octl() { return d_octl.as<KState>(); }
    BDev outer_view();
    template <typename T, typename Ti>
    void start_mixed(double alpha, double conv);
    template <typename T, typename Ti>
    void queue_inner(int todo);
    template <typename T, typename Ti>
    void queue_outer_step();
    template <typename Ti>
    void inner_setup();
    template <typename Ti>
    void precond32(const Ti *r, Ti *z, const KState *st);
    double conv_cri = 1.0e-8;
    std::vector<double> t_ms;  // set-up, iterations (ms) of the last solve
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};

    explicit Batch(int dev);
    ~Batch();
    int add(int n, int nnz, const int *rp, const int *ci, const double *val, int vt, int nrhs, const double *B);
    void clear();
    void set_rhs(int index, const double *B);
    std::vector<const void *> dev_rhs;  // right-hand sides to take from device memory at the next start
    void set_rhs_device(int index, const void *dB);
    void result_device(int index, void *dX);
    void update_values_device(int index, const void *dval);  // same pattern, new values (device memory)
    void assemble();
    BDev dev_view();
    KState *ctl();
    template <typename T>
    void start(int method_, double alpha, double conv, int max_ite_);
    template <typename T>
    void queue_chunk();
    bool poll();  // true when finished
    void wait();
    bool step();  // waits for the iterations in flight, queues more; true when finished
    // CUDA graph of GRAPH_ITERS iterations, captured once per start and replayed for
    // every whole group of that many iterations (not while profiling)
    static constexpr int GRAPH_ITERS = 8;
    bool use_graphs = true;
    // persistent ICCG (one CTA per instance runs all its iterations, ss_batch.cu): used
    // for FP64 ICCG starts when on (the default) and every instance has at most 8 tiles;
    // the same bits as the launches, 1.24x their speed on 1,024 instances of 1-4k rows
    bool persist = true;
    std::vector<int> h_sys_tile;        // host copy of the first tile of each instance
    DBuf d_pl_f, d_pr_f, d_pl_b, d_pr_b;  // per-instance level ranges of the forward / backward triangles
    uint64_t pr_key = ~0ull;            // pattern the ranges were made for
    bool persist_ok() const;
    void persist_ranges();
    template <typename T>
    void queue_persistent();
    cudaGraphExec_t graph_exec = nullptr;
    long long graph_kernels = 0;
    void drop_graph();
    template <typename F>
    void run_iterations(int todo, F &&issue_one);
    bool finished(int index) const;  // every instance of system `index` ended (as of the last completed chunk)
    // instance states as of the last completed chunk (the pinned copies are refilled by the next one)
    std::vector<KState> seen_st;
    std::vector<OState> seen_ost;
    cudaStream_t side = nullptr;  // copies of finished results while the batch runs
    int result(int index, double *X, int *iters, int *status);
    int residual_log(int index, int rhs, double *out, int capacity, int *length);
    int instance(int index, int rhs) const;
};

// settings a batch solves as the single-system path would: ICCG or IC-MRTR, a fixed
// accel_factor > 0, x0 = 0, the |b| normaliser, no diagonal scaling
bool batch_takes(const ssg_options &o, int method);
// nrhs right-hand sides of the handle's matrix (d_B, d_X: nrhs vectors of n values) in a
// one-system batch built from that matrix, kept while its version and nrhs are unchanged;
// iters / status (nullable) per right-hand side, status SSG_OK or SSG_NOT_CONVERGED
int solve_batched(Handle &h, Batch *&mb, uint64_t &mver, uint64_t &mpat, int precision, int method, double conv,
                  int max_ite, int nrhs, const void *d_B, void *d_X, int *iters, int *status);
// ssg_solve / ssg_solve_device with precision SSG_PREC_MIXED: the batch above, one right-hand side
int solve_mixed(Handle &h, Batch *&mb, uint64_t &mver, uint64_t &mpat, int method, double conv, int max_ite,
                const void *d_b, void *d_x);

template <typename F>
void Batch::run_iterations(int todo, F &&issue_one) {
    cudaStream_t s = h.stream;
    if (!use_graphs || h.prof.on || todo < GRAPH_ITERS || todo % GRAPH_ITERS != 0) {
        for (int c = 0; c < todo; ++c) issue_one();
        return;
    }
    if (!graph_exec) {
        cudaGraph_t g = nullptr;
        const long long l0 = launch_count();
        SSG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        try {
            for (int c = 0; c < GRAPH_ITERS; ++c) issue_one();
        } catch (...) {
            cudaStreamEndCapture(s, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        SSG_CUDA(cudaStreamEndCapture(s, &g));
        const cudaError_t e = cudaGraphInstantiate(&graph_exec, g, 0);
        cudaGraphDestroy(g);
        graph_kernels = launch_count() - l0;
        add_launches(-graph_kernels);  // captured, not run
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            graph_exec = nullptr;
            use_graphs = false;
            for (int c = 0; c < todo; ++c) issue_one();
            return;
        }
    }
    for (int k = 0; k < todo / GRAPH_ITERS; ++k) {
        SSG_CUDA(cudaGraphLaunch(graph_exec, s));
        add_launches(graph_kernels);
    }
}

}  // namespace ssg
