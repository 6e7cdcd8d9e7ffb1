// ss_capi.cu -- the extern "C" entry points declared in include/sparsesolv_gb300.h.
#include <cstring>
#include <new>

#include "ss_batch.cuh"
#include "ss_solver.cuh"

using ssg::cplx;
using ssg::Error;
using ssg::Handle;


struct ssg_handle_s {
    Handle *h;
    ssg::DBuf io_b, io_x;
    // one-system batch over this handle's matrix: mixed-precision solves and
    // several right-hand sides at once (ssg_solve_multi)
    ssg::Batch *ibatch = nullptr;
    uint64_t ib_version = ~0ull, ib_pattern = ~0ull;
};

namespace {

template <typename F>
int guarded(ssg_handle hd, F &&f) {
    if (!hd || !hd->h) return SSG_ERR_ARG;
    try {
        SSG_CUDA(cudaSetDevice(hd->h->device));
        ssg::AllocStream as(hd->h->stream);
        return f(*hd->h);
    } catch (const Error &e) {
        hd->h->last_error = e.msg;
        return e.code;
    } catch (const std::bad_alloc &) {
        hd->h->last_error = "host allocation failed";
        return SSG_ERR_NOMEM;
    }
}

size_t vbytes(const Handle &h) { return h.vtype == SSG_COMPLEX ? 16 : 8; }

}  // namespace

struct ssg_batch_s {
    ssg::Batch *b;
    std::string err;
};

namespace {

template <typename F>
int bguarded(ssg_batch bd, F &&f) {
    if (!bd || !bd->b) return SSG_ERR_ARG;
    try {
        SSG_CUDA(cudaSetDevice(bd->b->h.device));
        ssg::AllocStream as(bd->b->h.stream);
        return f(*bd->b);
    } catch (const Error &e) {
        bd->err = e.msg;
        return e.code;
    } catch (const std::bad_alloc &) {
        bd->err = "host allocation failed";
        return SSG_ERR_NOMEM;
    }
}

}  // namespace

extern "C" {

void ssg_default_options(ssg_options *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    // src/MatSolverBase.cpp:32-47
    o->is_init = 1;
    o->is_diag_scale = 0;
    o->is_save_best = 0;
    o->is_save_residual_log = 0;
    o->diverge_judge_type = 0;
    o->bad_div_val = 1000.0;
    o->bad_div_count_thres = 1000;
    o->conv_normalize_type = 0;
    o->conv_normalize_const = 1.0;
    // include/SparseSolv/MatSolverICCG.hpp:40, MatSolverMRTR.hpp:40-43
    o->accel_factor = 1.05;
    o->precondition_type = 1;
    o->precision = SSG_PREC_FP64;
    o->mrtr_reference_quirks = 0;
}

int ssg_create(ssg_handle *out, int device) {
    if (!out) return SSG_ERR_ARG;
    *out = nullptr;
    ssg_handle_s *hd = new (std::nothrow) ssg_handle_s();
    if (!hd) return SSG_ERR_NOMEM;
    try {
        hd->h = new Handle(device);
    } catch (const Error &e) {
        delete hd;
        return e.code;
    } catch (const std::bad_alloc &) {
        delete hd;
        return SSG_ERR_NOMEM;
    }
    *out = hd;
    return SSG_OK;
}

int ssg_destroy(ssg_handle hd) {
    if (!hd) return SSG_ERR_ARG;
    if (hd->h) cudaSetDevice(hd->h->device);
    hd->io_b.release();  // freed on the handle's stream, which lives until delete hd->h
    hd->io_x.release();
    delete hd->ibatch;
    delete hd->h;
    delete hd;
    return SSG_OK;
}

const char *ssg_last_error(ssg_handle hd) {
    if (!hd || !hd->h) return "invalid handle";
    return hd->h->last_error.c_str();
}

int ssg_set_options(ssg_handle hd, const ssg_options *o) {
    if (!o) return SSG_ERR_ARG;
    if (o->precision != SSG_PREC_FP64 && o->precision != SSG_PREC_MIXED) return SSG_ERR_ARG;
    return guarded(hd, [&](Handle &h) {
        h.opt = *o;
        return SSG_OK;
    });
}

int ssg_set_matrix(ssg_handle hd, int n, int nnz, const int32_t *row_ptr, const int32_t *col, const double *val,
                   int value_type) {
    if (!row_ptr || (nnz > 0 && (!col || !val))) return SSG_ERR_ARG;
    return guarded(hd, [&](Handle &h) {
        h.set_matrix(n, nnz, row_ptr, col, val, value_type, cudaMemcpyHostToDevice);
        return SSG_OK;
    });
}

int ssg_set_matrix_device(ssg_handle hd, int n, int nnz, const int32_t *row_ptr, const int32_t *col,
                          const double *val, int value_type) {
    if (!row_ptr || (nnz > 0 && (!col || !val))) return SSG_ERR_ARG;
    return guarded(hd, [&](Handle &h) {
        h.set_matrix(n, nnz, row_ptr, col, val, value_type, cudaMemcpyDeviceToDevice);
        return SSG_OK;
    });
}

static int check_solve_args(const Handle &h, int method, int max_ite) {
    if (h.vtype < 0) return SSG_ERR_STATE;
    if (method != SSG_METHOD_ICCG && method != SSG_METHOD_MRTR) return SSG_ERR_ARG;
    if (max_ite < 0) return SSG_ERR_ARG;
    return SSG_OK;
}

int ssg_solve_device(ssg_handle hd, int method, double conv_cri, int max_ite, double normB, const double *d_b,
                     double *d_x) {
    return guarded(hd, [&](Handle &h) {
        const int rc = check_solve_args(h, method, max_ite);
        if (rc) return rc;
        if (h.n > 0 && (!d_b || !d_x)) return SSG_ERR_ARG;
        if (h.opt.precision == SSG_PREC_MIXED)
            return ssg::solve_mixed(h, hd->ibatch, hd->ib_version, hd->ib_pattern, method, conv_cri, max_ite, d_b, d_x);
        if (h.vtype == SSG_COMPLEX) return h.solve<cplx>(method, conv_cri, max_ite, normB, (const cplx *)d_b, (cplx *)d_x);
        return h.solve<double>(method, conv_cri, max_ite, normB, d_b, d_x);
    });
}

int ssg_solve(ssg_handle hd, int method, double conv_cri, int max_ite, double normB, const double *b, double *x) {
    return guarded(hd, [&](Handle &h) {
        const int rc = check_solve_args(h, method, max_ite);
        if (rc) return rc;
        if (h.n > 0 && (!b || !x)) return SSG_ERR_ARG;
        const size_t bytes = vbytes(h) * (size_t)h.n;
        hd->io_b.ensure(bytes + 16);
        hd->io_x.ensure(bytes + 16);
        if (bytes) {
            SSG_CUDA(cudaMemcpyAsync(hd->io_b.p, b, bytes, cudaMemcpyHostToDevice, h.stream));
            SSG_CUDA(cudaMemcpyAsync(hd->io_x.p, x, bytes, cudaMemcpyHostToDevice, h.stream));
        }
        int res;
        if (h.opt.precision == SSG_PREC_MIXED)
            res = ssg::solve_mixed(h, hd->ibatch, hd->ib_version, hd->ib_pattern, method, conv_cri, max_ite, hd->io_b.p, hd->io_x.p);
        else if (h.vtype == SSG_COMPLEX)
            res = h.solve<cplx>(method, conv_cri, max_ite, normB, hd->io_b.as<cplx>(), hd->io_x.as<cplx>());
        else
            res = h.solve<double>(method, conv_cri, max_ite, normB, hd->io_b.as<double>(), hd->io_x.as<double>());
        if (bytes) SSG_CUDA(cudaMemcpyAsync(x, hd->io_x.p, bytes, cudaMemcpyDeviceToHost, h.stream));
        SSG_CUDA(cudaStreamSynchronize(h.stream));
        return res;
    });
}

// n_rhs right-hand sides: in the internal batch when its settings allow (one factor,
// shared launches), else one after another exactly as ssg_solve_device
static int solve_multi(ssg_handle hd, Handle &h, int method, double conv, int max_ite, int nrhs, const void *d_B,
                       void *d_X, int *iters, int *status) {
    const bool batched = ssg::batch_takes(h.opt, method) && !h.opt.is_save_best && h.opt.diverge_judge_type == 0;
    if (nrhs > 1 && h.n > 0 && batched)
        return ssg::solve_batched(h, hd->ibatch, hd->ib_version, hd->ib_pattern, h.opt.precision, method, conv,
                                  max_ite, nrhs, d_B, d_X, iters, status);
    const size_t vb = vbytes(h) * (size_t)h.n;
    int all = SSG_OK;
    for (int k = 0; k < nrhs; ++k) {
        const char *b = (const char *)d_B + vb * k;
        char *x = (char *)d_X + vb * k;
        int r;
        if (h.opt.precision == SSG_PREC_MIXED)
            r = ssg::solve_mixed(h, hd->ibatch, hd->ib_version, hd->ib_pattern, method, conv, max_ite, b, x);
        else if (h.vtype == SSG_COMPLEX)
            r = h.solve<cplx>(method, conv, max_ite, -1.0, (const cplx *)b, (cplx *)x);
        else
            r = h.solve<double>(method, conv, max_ite, -1.0, (const double *)b, (double *)x);
        if (iters) iters[k] = h.iters;
        if (status) status[k] = r;
        if (r != SSG_OK) all = SSG_NOT_CONVERGED;
    }
    return all;
}

int ssg_solve_multi_device(ssg_handle hd, int method, double conv_cri, int max_ite, int n_rhs, const double *d_B,
                           double *d_X, int *iters, int *status) {
    return guarded(hd, [&](Handle &h) {
        const int rc = check_solve_args(h, method, max_ite);
        if (rc) return rc;
        if (n_rhs < 0 || (h.n > 0 && n_rhs > 0 && (!d_B || !d_X))) return SSG_ERR_ARG;
        return solve_multi(hd, h, method, conv_cri, max_ite, n_rhs, d_B, d_X, iters, status);
    });
}

int ssg_solve_multi(ssg_handle hd, int method, double conv_cri, int max_ite, int n_rhs, const double *B, double *X,
                    int *iters, int *status) {
    return guarded(hd, [&](Handle &h) {
        const int rc = check_solve_args(h, method, max_ite);
        if (rc) return rc;
        if (n_rhs < 0 || (h.n > 0 && n_rhs > 0 && (!B || !X))) return SSG_ERR_ARG;
        const size_t bytes = vbytes(h) * (size_t)h.n * (size_t)n_rhs;
        hd->io_b.ensure(bytes + 16);
        hd->io_x.ensure(bytes + 16);
        if (bytes) {
            SSG_CUDA(cudaMemcpyAsync(hd->io_b.p, B, bytes, cudaMemcpyHostToDevice, h.stream));
            SSG_CUDA(cudaMemcpyAsync(hd->io_x.p, X, bytes, cudaMemcpyHostToDevice, h.stream));
        }
        const int res = solve_multi(hd, h, method, conv_cri, max_ite, n_rhs, hd->io_b.p, hd->io_x.p, iters, status);
        if (bytes) SSG_CUDA(cudaMemcpyAsync(X, hd->io_x.p, bytes, cudaMemcpyDeviceToHost, h.stream));
        SSG_CUDA(cudaStreamSynchronize(h.stream));
        return res;
    });
}

int ssg_set_matrix_coo(ssg_handle hd, int n, int nnz, const int32_t *rows, const int32_t *cols, const double *vals,
                       int value_type, int on_device) {
    if (nnz > 0 && (!rows || !cols || !vals)) return SSG_ERR_ARG;
    return guarded(hd, [&](Handle &h) {
        h.set_matrix_coo(n, nnz, rows, cols, vals, value_type,
                         on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice);
        return SSG_OK;
    });
}

int ssg_flux_density(ssg_handle hd, int nx, int ny, int nz, double hx, double hy, double hz, const int32_t *ex,
                     const int32_t *ey, const int32_t *ez, int nunk, const void *A, int value_type, void *B,
                     int on_device) {
    if (!ex || !ey || !ez || !B || (nunk > 0 && !A)) return SSG_ERR_ARG;
    return guarded(hd, [&](Handle &h) {
        ssg::flux_density_any(h, nx, ny, nz, hx, hy, hz, ex, ey, ez, nunk, A, value_type, B, on_device != 0);
        return SSG_OK;
    });
}

int ssg_set_matrix_voxel(ssg_handle hd, int nx, int ny, int nz, const int32_t *ex, const int32_t *ey,
                         const int32_t *ez, int nunk, const double *Ke, const double *Me, const double *Ce,
                         const double *nu, const double *sig, double omega, const double *tz, int value_type, void *b,
                         int on_device) {
    return guarded(hd, [&](Handle &h) {
        ssg::voxel_assemble_any(h, nx, ny, nz, ex, ey, ez, nunk, Ke, Me, Ce, nu, sig, omega, tz, value_type, b,
                                on_device != 0);
        return SSG_OK;
    });
}

int ssg_get_matrix(ssg_handle hd, int32_t *row_ptr, int32_t *col, double *val, int *n, int *nnz) {
    return guarded(hd, [&](Handle &h) {
        if (h.vtype < 0) return SSG_ERR_STATE;
        if (n) *n = h.n;
        if (nnz) *nnz = h.nnz;
        if (row_ptr)
            SSG_CUDA(cudaMemcpyAsync(row_ptr, h.A_rp.p, sizeof(int) * ((size_t)h.n + 1), cudaMemcpyDeviceToHost,
                                     h.stream));
        if (col && h.nnz)
            SSG_CUDA(cudaMemcpyAsync(col, h.A_ci.p, sizeof(int) * (size_t)h.nnz, cudaMemcpyDeviceToHost, h.stream));
        if (val && h.nnz)
            SSG_CUDA(cudaMemcpyAsync(val, h.A_val.p, vbytes(h) * (size_t)h.nnz, cudaMemcpyDeviceToHost, h.stream));
        SSG_CUDA(cudaStreamSynchronize(h.stream));
        return SSG_OK;
    });
}

int ssg_update_values(ssg_handle hd, const double *val) {
    return guarded(hd, [&](Handle &h) {
        if (h.nnz > 0 && !val) return SSG_ERR_ARG;
        h.update_values(val, cudaMemcpyHostToDevice);
        return SSG_OK;
    });
}

int ssg_update_values_device(ssg_handle hd, const double *d_val) {
    return guarded(hd, [&](Handle &h) {
        if (h.nnz > 0 && !d_val) return SSG_ERR_ARG;
        h.update_values(d_val, cudaMemcpyDeviceToDevice);
        return SSG_OK;
    });
}

int ssg_get_stream(ssg_handle hd, void **stream) {
    if (!stream) return SSG_ERR_ARG;
    return guarded(hd, [&](Handle &h) {
        *stream = (void *)h.stream;
        return SSG_OK;
    });
}

static void prof_reset(Handle &h, bool on) {
    h.prof.on = on;
    for (int c = 0; c < ssg::PC_N; ++c) {
        h.prof.ms[c] = 0.0;
        h.prof.launches[c] = 0;
        h.prof.bytes[c] = 0.0;
    }
    h.prof.recs.clear();
    h.prof.used = 0;
}

int ssg_set_profiling(ssg_handle hd, int enable) {
    return guarded(hd, [&](Handle &h) {
        prof_reset(h, enable != 0);
        if (hd->ibatch) prof_reset(hd->ibatch->h, enable != 0);
        return SSG_OK;
    });
}

int ssg_get_kernel_stats(ssg_handle hd, double *ms, long long *launches, double *bytes, int cap) {
    return guarded(hd, [&](Handle &h) {
        // mixed-precision and multi-right-hand-side solves run in the handle's internal batch:
        // its launches count too
        const Handle *mh = hd->ibatch ? &hd->ibatch->h : nullptr;
        for (int c = 0; c < ssg::PC_N && c < cap; ++c) {
            if (ms) ms[c] = h.prof.ms[c] + (mh ? mh->prof.ms[c] : 0.0);
            if (launches) launches[c] = h.prof.launches[c] + (mh ? mh->prof.launches[c] : 0);
            if (bytes) bytes[c] = h.prof.bytes[c] + (mh ? mh->prof.bytes[c] : 0.0);
        }
        return SSG_OK;
    });
}

long long ssg_launch_count(void) { return ssg::launch_count(); }

int ssg_autotune(ssg_handle hd, int keep_group, int *mode, int *group, int *cta_per_sm, double *ms) {
    return guarded(hd, [&](Handle &h) {
        const Handle::TuneChoice c =
            h.vtype == SSG_COMPLEX ? h.autotune<cplx>(keep_group != 0) : h.autotune<double>(keep_group != 0);
        if (mode) *mode = c.mode;
        if (group) *group = c.group;
        if (cta_per_sm) *cta_per_sm = c.cta_per_sm;
        if (ms) *ms = c.ms;
        return SSG_OK;
    });
}

int ssg_set_tuning(ssg_handle hd, int key, int value) {
    return guarded(hd, [&](Handle &h) {
        switch (key) {
            case SSG_TUNE_SWEEP_CTA_PER_SM:
                if (value < 0 || value > 32) return SSG_ERR_ARG;
                h.swcfg.cta_per_sm = value;
                break;
            case SSG_TUNE_SWEEP_GROUP:
                if (value != 0 && value != 4 && value != 8 && value != 16 && value != 32) return SSG_ERR_ARG;
                h.swcfg.group = value;
                break;
            case SSG_TUNE_SWEEP_BACKOFF_NS:
                if (value < 0 || value > 100000) return SSG_ERR_ARG;
                h.swcfg.backoff_ns = value;
                break;
            case SSG_TUNE_FACTOR_BACKOFF_NS:
                if (value < 0 || value > 100000) return SSG_ERR_ARG;
                h.fac_backoff_ns = value;
                break;
            case SSG_TUNE_RECIPROCAL_DIAG:
                h.use_inv_diag = value != 0;
                break;
            case SSG_TUNE_SWEEP_MODE:
                if (value < 0 || value > 4) return SSG_ERR_ARG;
                h.sweep_mode = value;
                break;
            case SSG_TUNE_CLUSTER_RING_KB:
                if (value < 4 || value > 200) return SSG_ERR_ARG;
                h.cl_ring_bytes = value * 1024;
                break;
            case SSG_TUNE_CLUSTER_GROUP:
                if (value != 4 && value != 8 && value != 16 && value != 32) return SSG_ERR_ARG;
                h.cl_group = value;
                break;
            case SSG_TUNE_SPMV_GROUP:
                if (value != 0 && value != 2 && value != 4 && value != 8 && value != 16 && value != 32) return SSG_ERR_ARG;
                h.spmv_group_req = value;
                break;
            case SSG_TUNE_BATCH_GROUP:
                if (value != 0 && value != 4 && value != 8 && value != 16) return SSG_ERR_ARG;
                h.batch_group = value;
                break;
            case SSG_TUNE_SPIN_LIMIT_US:
                if (value < 0) return SSG_ERR_ARG;
                h.set_spin_limit(value);
                break;
            default:
                return SSG_ERR_ARG;
        }
        return SSG_OK;
    });
}

int ssg_get_residual_log(ssg_handle hd, double *log, int cap, int *len) {
    return guarded(hd, [&](Handle &h) {
        // MatSolverBase::getResidualLog: zeros of the stored size when logging is off
        const int sz = (int)h.residual_log.size();
        if (len) *len = sz;
        if (log)
            for (int i = 0; i < sz && i < cap; ++i) log[i] = h.opt.is_save_residual_log ? h.residual_log[i] : 0.0;
        return SSG_OK;
    });
}

int ssg_get_iters(ssg_handle hd, int *iters) {
    if (!iters) return SSG_ERR_ARG;
    return guarded(hd, [&](Handle &h) {
        *iters = h.iters;
        return SSG_OK;
    });
}

int ssg_get_accel_used(ssg_handle hd, double *alpha) {
    if (!alpha) return SSG_ERR_ARG;
    return guarded(hd, [&](Handle &h) {
        *alpha = h.alpha_used;
        return SSG_OK;
    });
}

int ssg_get_timings(ssg_handle hd, double *ms, int cap) {
    if (!ms) return SSG_ERR_ARG;
    return guarded(hd, [&](Handle &h) {
        if (cap > 0) ms[0] = h.t_setup_ms;
        if (cap > 1) ms[1] = h.t_iter_ms;
        return SSG_OK;
    });
}

int ssg_factor(ssg_handle hd, double alpha, int32_t *lrp, int32_t *lci, double *lval, double *D, int *nnzL) {
    return guarded(hd, [&](Handle &h) {
        if (h.vtype < 0) return SSG_ERR_STATE;
        const size_t vb = vbytes(h);
        if (h.vtype == SSG_COMPLEX)
            h.ensure_factor<cplx>(alpha, false);
        else
            h.ensure_factor<double>(alpha, false);
        if (nnzL) *nnzL = h.nnzL;
        ssg::DBuf nat;
        nat.alloc(vb * (size_t)(h.nnzL + 1));
        if (h.vtype == SSG_COMPLEX)
            ssg::gather_values<cplx>(h.nat2lev.as<int>(), h.Lval.as<cplx>(), nat.as<cplx>(), h.nnzL, h.stream);
        else
            ssg::gather_values<double>(h.nat2lev.as<int>(), h.Lval.as<double>(), nat.as<double>(), h.nnzL, h.stream);
        if (lrp) SSG_CUDA(cudaMemcpyAsync(lrp, h.Lnat_rp.p, sizeof(int) * (size_t)(h.n + 1), cudaMemcpyDeviceToHost, h.stream));
        if (lci && h.nnzL)
            SSG_CUDA(cudaMemcpyAsync(lci, h.Lnat_ci.p, sizeof(int) * (size_t)h.nnzL, cudaMemcpyDeviceToHost, h.stream));
        if (lval && h.nnzL) SSG_CUDA(cudaMemcpyAsync(lval, nat.p, vb * (size_t)h.nnzL, cudaMemcpyDeviceToHost, h.stream));
        if (D && h.n) SSG_CUDA(cudaMemcpyAsync(D, h.Dvec.p, vb * (size_t)h.n, cudaMemcpyDeviceToHost, h.stream));
        SSG_CUDA(cudaStreamSynchronize(h.stream));
        return SSG_OK;
    });
}

int ssg_apply_precond(ssg_handle hd, const double *r, double *z) {
    return guarded(hd, [&](Handle &h) {
        if (!h.fac_valid || h.fac_version != h.version) return SSG_ERR_STATE;
        const size_t bytes = vbytes(h) * (size_t)h.n;
        h.ensure_work(vbytes(h));
        hd->io_b.ensure(bytes + 16);
        hd->io_x.ensure(bytes + 16);
        SSG_CUDA(cudaMemcpyAsync(hd->io_b.p, r, bytes, cudaMemcpyHostToDevice, h.stream));
        if (h.vtype == SSG_COMPLEX)
            h.apply_precond<cplx>(hd->io_b.as<cplx>(), hd->io_x.as<cplx>(), nullptr);
        else
            h.apply_precond<double>(hd->io_b.as<double>(), hd->io_x.as<double>(), nullptr);
        SSG_CUDA(cudaMemcpyAsync(z, hd->io_x.p, bytes, cudaMemcpyDeviceToHost, h.stream));
        SSG_CUDA(cudaStreamSynchronize(h.stream));
        h.check_err("preconditioner");
        return SSG_OK;
    });
}

int ssg_spmv(ssg_handle hd, const double *x, double *y) {
    return guarded(hd, [&](Handle &h) {
        if (h.vtype < 0) return SSG_ERR_STATE;
        const size_t bytes = vbytes(h) * (size_t)h.n;
        hd->io_b.ensure(bytes + 16);
        hd->io_x.ensure(bytes + 16);
        SSG_CUDA(cudaMemcpyAsync(hd->io_b.p, x, bytes, cudaMemcpyHostToDevice, h.stream));
        if (h.vtype == SSG_COMPLEX)
            ssg::spmv<cplx>(h.n, h.spmv_lanes(), h.A_rp.as<int>(), h.A_ci.as<int>(), h.A_val.as<cplx>(), hd->io_b.as<cplx>(),
                            hd->io_x.as<cplx>(), h.stream);
        else
            ssg::spmv<double>(h.n, h.spmv_lanes(), h.A_rp.as<int>(), h.A_ci.as<int>(), h.A_val.as<double>(), hd->io_b.as<double>(),
                              hd->io_x.as<double>(), h.stream);
        SSG_CUDA(cudaMemcpyAsync(y, hd->io_x.p, bytes, cudaMemcpyDeviceToHost, h.stream));
        SSG_CUDA(cudaStreamSynchronize(h.stream));
        return SSG_OK;
    });
}

int ssg_level_schedule(ssg_handle hd, int lower, int32_t *level, int32_t *perm, int *nlev) {
    return guarded(hd, [&](Handle &h) {
        if (h.vtype < 0) return SSG_ERR_STATE;
        h.ensure_patterns(false, !lower);
        const ssg::Tri &T = lower ? h.Lf : h.Ub;
        if (nlev) *nlev = T.nlev;
        if (level && h.n)
            SSG_CUDA(cudaMemcpyAsync(level, T.level.p, sizeof(int) * (size_t)h.n, cudaMemcpyDeviceToHost, h.stream));
        if (perm && h.n)
            SSG_CUDA(cudaMemcpyAsync(perm, T.perm.p, sizeof(int) * (size_t)h.n, cudaMemcpyDeviceToHost, h.stream));
        SSG_CUDA(cudaStreamSynchronize(h.stream));
        return SSG_OK;
    });
}

int ssg_batch_create(ssg_batch *out, int device) {
    if (!out) return SSG_ERR_ARG;
    *out = nullptr;
    ssg_batch_s *bd = new (std::nothrow) ssg_batch_s();
    if (!bd) return SSG_ERR_NOMEM;
    try {
        bd->b = new ssg::Batch(device);
    } catch (const Error &e) {
        delete bd;
        return e.code;
    } catch (const std::bad_alloc &) {
        delete bd;
        return SSG_ERR_NOMEM;
    }
    *out = bd;
    return SSG_OK;
}

int ssg_batch_destroy(ssg_batch bd) {
    if (!bd) return SSG_ERR_ARG;
    if (bd->b) {
        cudaSetDevice(bd->b->h.device);
        if (bd->b->running) cudaStreamSynchronize(bd->b->h.stream);
        delete bd->b;
    }
    delete bd;
    return SSG_OK;
}

const char *ssg_batch_last_error(ssg_batch bd) { return bd ? bd->err.c_str() : "null batch"; }

int ssg_batch_add(ssg_batch bd, int n, int nnz, const int32_t *rp, const int32_t *ci, const void *val, int value_type,
                  int n_rhs, const void *B, int *index) {
    return bguarded(bd, [&](ssg::Batch &b) {
        const int i = b.add(n, nnz, rp, ci, (const double *)val, value_type, n_rhs, (const double *)B);
        if (index) *index = i;
        return SSG_OK;
    });
}

int ssg_batch_set_rhs(ssg_batch bd, int index, const void *B) {
    return bguarded(bd, [&](ssg::Batch &b) {
        b.set_rhs(index, (const double *)B);
        return SSG_OK;
    });
}

int ssg_batch_clear(ssg_batch bd) {
    return bguarded(bd, [&](ssg::Batch &b) {
        b.clear();
        return SSG_OK;
    });
}

int ssg_batch_start(ssg_batch bd, int method, double alpha, double conv, int max_ite) {
    return bguarded(bd, [&](ssg::Batch &b) {
        if (b.sys.empty()) return SSG_ERR_STATE;
        if (b.vtype == SSG_COMPLEX)
            b.start<cplx>(method, alpha, conv, max_ite);
        else
            b.start<double>(method, alpha, conv, max_ite);
        return SSG_OK;
    });
}

int ssg_batch_poll(ssg_batch bd, int *done) {
    return bguarded(bd, [&](ssg::Batch &b) {
        const bool d = b.poll();
        if (done) *done = d ? 1 : 0;
        return SSG_OK;
    });
}

int ssg_batch_step(ssg_batch bd, int *done) {
    return bguarded(bd, [&](ssg::Batch &b) {
        const bool d = b.step();
        if (done) *done = d ? 1 : 0;
        return SSG_OK;
    });
}

int ssg_batch_finished(ssg_batch bd, int index, int *finished) {
    return bguarded(bd, [&](ssg::Batch &b) {
        const bool f = b.finished(index);
        if (finished) *finished = f ? 1 : 0;
        return SSG_OK;
    });
}

int ssg_batch_wait(ssg_batch bd) {
    return bguarded(bd, [&](ssg::Batch &b) {
        b.wait();
        return SSG_OK;
    });
}

int ssg_batch_result(ssg_batch bd, int index, void *X, int *iters, int *status) {
    return bguarded(bd, [&](ssg::Batch &b) { return b.result(index, (double *)X, iters, status); });
}

int ssg_batch_residual_log(ssg_batch bd, int index, int rhs, double *log, int capacity, int *length) {
    return bguarded(bd, [&](ssg::Batch &b) { return b.residual_log(index, rhs, log, capacity, length); });
}

int ssg_batch_timings(ssg_batch bd, double *ms2) {
    return bguarded(bd, [&](ssg::Batch &b) {
        if (!ms2) return SSG_ERR_ARG;
        ms2[0] = b.t_ms.size() > 0 ? b.t_ms[0] : 0.0;
        ms2[1] = b.t_ms.size() > 1 ? b.t_ms[1] : 0.0;
        return SSG_OK;
    });
}

int ssg_batch_set_precision(ssg_batch bd, int precision, double inner_tol) {
    return bguarded(bd, [&](ssg::Batch &b) {
        if (precision != SSG_PREC_FP64 && precision != SSG_PREC_MIXED) return SSG_ERR_ARG;
        if (b.running) return SSG_ERR_STATE;
        if (inner_tol >= 1.0) return SSG_ERR_ARG;
        b.precision = precision;
        b.inner_tol = inner_tol > 0.0 ? inner_tol : 0.0;
        return SSG_OK;
    });
}

int ssg_batch_set_graphs(ssg_batch bd, int enable) {
    return bguarded(bd, [&](ssg::Batch &b) {
        if (b.running) return SSG_ERR_STATE;
        b.use_graphs = enable != 0;
        b.drop_graph();
        return SSG_OK;
    });
}

int ssg_batch_set_persistent(ssg_batch bd, int enable) {
    return bguarded(bd, [&](ssg::Batch &b) {
        if (b.running) return SSG_ERR_STATE;
        b.persist = enable != 0;
        return SSG_OK;
    });
}

int ssg_batch_autotune(ssg_batch bd, int *mode, int *group, int *cta_per_sm, double *ms) {
    return bguarded(bd, [&](ssg::Batch &b) {
        if (b.running) return SSG_ERR_STATE;
        if (!b.assembled) b.assemble();
        // the batch engine runs its own sweeps (sync-free and one-cluster), not the push sweep
        const Handle::TuneChoice c =
            b.vtype == SSG_COMPLEX ? b.h.autotune<cplx>(false, false) : b.h.autotune<double>(false, false);
        b.drop_graph();  // the captured iterations used the previous schedule
        if (mode) *mode = c.mode;
        if (group) *group = c.group;
        if (cta_per_sm) *cta_per_sm = c.cta_per_sm;
        if (ms) *ms = c.ms;
        return SSG_OK;
    });
}

int ssg_batch_set_profiling(ssg_batch bd, int enable) {
    return bguarded(bd, [&](ssg::Batch &b) {
        Handle &h = b.h;
        h.prof.on = enable != 0;
        for (int c = 0; c < ssg::PC_N; ++c) {
            h.prof.ms[c] = 0.0;
            h.prof.launches[c] = 0;
            h.prof.bytes[c] = 0.0;
        }
        h.prof.recs.clear();
        h.prof.used = 0;
        return SSG_OK;
    });
}

int ssg_batch_kernel_stats(ssg_batch bd, double *ms, long long *launches, double *bytes, int cap) {
    return bguarded(bd, [&](ssg::Batch &b) {
        for (int c = 0; c < ssg::PC_N && c < cap; ++c) {
            if (ms) ms[c] = b.h.prof.ms[c];
            if (launches) launches[c] = b.h.prof.launches[c];
            if (bytes) bytes[c] = b.h.prof.bytes[c];
        }
        return SSG_OK;
    });
}

int ssg_batch_stream(ssg_batch bd, void **stream) {
    return bguarded(bd, [&](ssg::Batch &b) {
        if (!stream) return SSG_ERR_ARG;
        *stream = (void *)b.h.stream;
        return SSG_OK;
    });
}

int ssg_ic_factor_noalloc(int n, int nnz, const int32_t *lrp, const int32_t *lci, const void *lower_val, void *lval,
                          void *D, double alpha, int value_type, void *stream) {
    return ssg::ic_factor_noalloc(n, nnz, lrp, lci, lower_val, lval, D, alpha, value_type, (cudaStream_t)stream);
}

}  // extern "C"
