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
    KState *ctl;          // batch control: active while any instance is
    double *part;         // [NT * BATCH_PARTS]
    unsigned *counter;    // last-block ticket
    double *logs;         // [S * log_stride] residual logs
    int log_stride;
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
    int S = 0, NT = 0;
    bool assembled = false;
    bool rhs_dirty = true;  // right-hand sides changed since the last upload
    DBuf d_tile, d_tile_sys, d_sys_tile, d_sys_row, d_st, d_part, d_logs, d_ctl_counter;
    KState *h_st = nullptr;   // pinned copy of the instance states
    KState *h_ctl = nullptr;  // pinned copy of the control state
    cudaEvent_t ev_chunk = nullptr;
    // the running solve
    int method = SSG_METHOD_ICCG;
    int max_ite = 0, queued = 0, chunk = 2, iter_no = 0;
    bool running = false, log_on = true;
    std::vector<double> t_ms;  // set-up, iterations (ms) of the last solve
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};

    explicit Batch(int dev);
    ~Batch();
    int add(int n, int nnz, const int *rp, const int *ci, const double *val, int vt, int nrhs, const double *B);
    void clear();
    void set_rhs(int index, const double *B);
    void assemble();
    BDev dev_view();
    KState *ctl();
    template <typename T>
    void start(int method_, double alpha, double conv, int max_ite_);
    template <typename T>
    void queue_chunk();
    bool poll();  // true when finished
    void wait();
    int result(int index, double *X, int *iters, int *status);
    int residual_log(int index, int rhs, double *out, int capacity, int *length);
    int instance(int index, int rhs) const;
};

}  // namespace ssg
