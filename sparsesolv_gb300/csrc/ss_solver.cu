// ss_solver.cu -- host orchestration of one solve() call on the device.
//
// Mirrors MatSolverICCG::solve / MatSolverMRTR::solve
// (src/MatSolverICCG.cpp:99-168, src/MatSolverMRTR_ICver.cpp:99-173,
// src/MatSolverMRTR_SGSver.cpp:42-69) with these GB300 choices:
//   - the matrix, its level schedules, the factor and all Krylov vectors stay
//     resident in HBM; the factor is reused while the matrix values, alpha and
//     the scaling mode are unchanged (the reference refactors on every call;
//     reuse returns the identical factor, so results do not change);
//   - the iteration runs entirely on the device: scalar recurrences,
//     convergence test, divergence judge and best tracking are evaluated by
//     the kernels (ss_spmv_vec.cu), the host queues chunks of iterations and
//     reads one status word between chunks.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "ss_solver.cuh"

namespace ssg {

Handle::Handle(int dev) : device(dev) {
    SSG_CUDA(cudaSetDevice(dev));
    SSG_CUDA(cudaStreamCreateWithFlags(&sg.s, cudaStreamNonBlocking));
    stream = sg.s;
    // stream-ordered allocations come from the device's default pool; keep what it
    // holds instead of returning it at every synchronisation (a per-process setting)
    static bool pool_set[64] = {};
    if (dev >= 0 && dev < 64 && !pool_set[dev]) {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        pool_set[dev] = true;
    }
    ssg_default_options(&opt);
    part.alloc(part_bytes());
    SSG_CUDA(cudaMemset(part.p, 0, part.bytes));
    state.alloc(sizeof(KState));
    SSG_CUDA(cudaMemset(state.p, 0, sizeof(KState)));
    small.alloc(256);
    SSG_CUDA(cudaMemset(small.p, 0, 256));
    SSG_CUDA(cudaMallocHost(&h_state, sizeof(KState)));
    SSG_CUDA(cudaMallocHost(&h_scal, 64 * sizeof(double)));
    for (auto &e : ev) SSG_CUDA(cudaEventCreate(&e));
}

int Handle::prof_begin(int cls) {
    if (!prof.on) return -1;
    if (prof.used + 2 > prof.pool.size()) {
        for (int k = 0; k < 64; ++k) {
            cudaEvent_t e;
            SSG_CUDA(cudaEventCreate(&e));
            prof.pool.push_back(e);
        }
    }
    ProfRec r{cls, prof.iter, prof.pre, prof.pool[prof.used], prof.pool[prof.used + 1], 0.0};
    prof.used += 2;
    SSG_CUDA(cudaEventRecord(r.a, stream));
    prof.recs.push_back(r);
    return (int)prof.recs.size() - 1;
}

void Handle::prof_end(int idx, double bytes) {
    if (idx < 0) return;
    prof.recs[idx].bytes = bytes;
    SSG_CUDA(cudaEventRecord(prof.recs[idx].b, stream));
}

// keep the launches that did work: set-up (iteration 0), every launch of the
// iterations before the last, and the pre-decision launches of the last one
void Handle::prof_flush(int iters_done) {
    if (!prof.on) return;
    SSG_CUDA(cudaStreamSynchronize(stream));
    for (const auto &r : prof.recs) {
        if (!(r.iter == 0 || r.iter < iters_done || (r.iter == iters_done && r.pre))) continue;
        float ms = 0.f;
        SSG_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        prof.ms[r.cls] += ms;
        prof.launches[r.cls] += 1;
        prof.bytes[r.cls] += r.bytes;
    }
    prof.recs.clear();
    prof.used = 0;
}

Handle::~Handle() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto e : prof.pool) cudaEventDestroy(e);
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    if (h_state) cudaFreeHost(h_state);
    if (h_scal) cudaFreeHost(h_scal);
    // the stream itself goes with sg, after the buffers have been freed on it
}

void Handle::set_spin_limit(int us) {
    spin_limit_us = us;
    SSG_CUDA(cudaMemcpyAsync(err() + 1, &spin_limit_us, sizeof(int), cudaMemcpyHostToDevice, stream));
    SSG_CUDA(cudaStreamSynchronize(stream));
}

void Handle::check_err(const char *where) {
    int herr = 0;
    SSG_CUDA(cudaMemcpyAsync(&herr, err(), sizeof(int), cudaMemcpyDeviceToHost, stream));
    SSG_CUDA(cudaStreamSynchronize(stream));
    if (herr == ERR_NONE) return;
    SSG_CUDA(cudaMemsetAsync(err(), 0, sizeof(int), stream));
    SSG_CUDA(cudaStreamSynchronize(stream));
    if (herr == ERR_TIMEOUT) throw Error{SSG_ERR_TIMEOUT, std::string(where) + ": a bounded device wait timed out"};
    if (herr == ERR_NO_DIAG) throw Error{SSG_ERR_NO_DIAGONAL, "there is not diagonal element!"};
    if (herr == ERR_PATTERN) throw Error{SSG_ERR_ARG, std::string(where) + ": bad column pattern"};
    if (herr == ERR_ROW_TOO_LONG)
        throw Error{SSG_ERR_ARG, std::string(where) + ": a row of the lower triangle is longer than the kernel takes"};
    throw Error{SSG_ERR_STATE, std::string(where) + ": device error " + std::to_string(herr)};
}

void Handle::set_matrix(int n_, int nnz_, const int32_t *rp, const int32_t *ci, const double *val, int vt,
                        cudaMemcpyKind kind) {
    if (n_ < 0 || nnz_ < 0 || (vt != SSG_REAL && vt != SSG_COMPLEX)) throw Error{SSG_ERR_ARG, "bad matrix arguments"};
    const size_t vb = (vt == SSG_COMPLEX ? 16 : 8);
    // a new pattern invalidates the schedules unless rp/ci are identical
    bool same_pattern = (n_ == n && nnz_ == nnz && pat_version != ~0ull);
    if (same_pattern) {
        // compare on the device would need another copy; compare host-side when the input is on the host
        if (kind == cudaMemcpyHostToDevice) {
            std::vector<int> hrp(n_ + 1), hci(nnz_);
            SSG_CUDA(cudaMemcpy(hrp.data(), A_rp.p, sizeof(int) * (n_ + 1), cudaMemcpyDeviceToHost));
            SSG_CUDA(cudaMemcpy(hci.data(), A_ci.p, sizeof(int) * nnz_, cudaMemcpyDeviceToHost));
            same_pattern = !memcmp(hrp.data(), rp, sizeof(int) * (n_ + 1)) && !memcmp(hci.data(), ci, sizeof(int) * nnz_);
        } else {
            same_pattern = false;
        }
    }
    n = n_;
    nnz = nnz_;
    vtype = vt;
    A_rp.ensure(sizeof(int) * (size_t)(n + 1));
    A_ci.ensure(sizeof(int) * (size_t)(nnz + 1));
    A_val.ensure(vb * (size_t)(nnz + 1));
    SSG_CUDA(cudaMemcpyAsync(A_rp.p, rp, sizeof(int) * (size_t)(n + 1), kind, stream));
    if (nnz) SSG_CUDA(cudaMemcpyAsync(A_ci.p, ci, sizeof(int) * (size_t)nnz, kind, stream));
    if (nnz) SSG_CUDA(cudaMemcpyAsync(A_val.p, val, vb * (size_t)nnz, kind, stream));
    SSG_CUDA(cudaStreamSynchronize(stream));
    ++version;
    if (!same_pattern) {
        ++pattern_id;
        pat_version = ~0ull;
        ltb_ready = ub_ready = false;
        note_row_lengths(kind == cudaMemcpyHostToDevice ? rp : nullptr);
    } else {
        pat_version = version;
    }
    fac_valid = sgs_valid = dad_valid = false;
}

// the SpMV's lanes a row follow the pattern's row-length distribution; rp on the host, or
// null to read the device copy
void Handle::note_row_lengths(const int32_t *host_rp) {
    if (host_rp) {
        spmv_len = spmv_rowlen(n, host_rp);
        return;
    }
    std::vector<int> hrp((size_t)n + 1);
    SSG_CUDA(cudaMemcpyAsync(hrp.data(), A_rp.p, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToHost, stream));
    SSG_CUDA(cudaStreamSynchronize(stream));
    spmv_len = spmv_rowlen(n, hrp.data());
}

void Handle::update_values(const double *val, cudaMemcpyKind kind) {
    if (vtype < 0) throw Error{SSG_ERR_STATE, "no matrix set"};
    const size_t vb = (vtype == SSG_COMPLEX ? 16 : 8);
    if (nnz) SSG_CUDA(cudaMemcpyAsync(A_val.p, val, vb * (size_t)nnz, kind, stream));
    SSG_CUDA(cudaStreamSynchronize(stream));
    values_changed();
}

void Handle::values_changed() {
    const bool pat_ok = (pat_version == version);
    ++version;
    if (pat_ok) pat_version = version;  // the pattern and its schedules stay valid
    fac_valid = sgs_valid = dad_valid = false;
}

void Handle::set_replicas(const std::vector<int> &src) {
    rep_on = false;
    for (int v : src)
        if (v >= 0) {
            rep_on = true;
            break;
        }
    if (rep_on) {
        if ((int)src.size() != n) throw Error{SSG_ERR_ARG, "replica map size"};
        rep_src.ensure(sizeof(int) * (size_t)(n + 1));
        SSG_CUDA(cudaMemcpyAsync(rep_src.p, src.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, stream));
        SSG_CUDA(cudaStreamSynchronize(stream));
    }
    fac_sub_valid = false;
    fac_valid = false;
}

void Handle::ensure_patterns(bool need_ltb, bool need_ub) {
    DBuf tmp;
    if (pat_version != version) {
        fac_sub_valid = false;
        triangle_pattern(n, A_rp.as<int>(), A_ci.as<int>(), true, Lnat_rp, Lnat_ci, Lnat_src, nnzL, stream, tmp);
        timed(PC_LEVELS, 0.0, [&] {
            build_tri(Lf, n, nnzL, Lnat_rp.as<int>(), Lnat_ci.as<int>(), Lnat_src.as<int>(), true, err(), stream, tmp);
        });
        check_err("level schedule");
        nat2lev.ensure(sizeof(int) * (size_t)(nnzL + 1));
        level_positions(Lf, Lnat_rp.as<int>(), nat2lev.as<int>(), stream);
        factor_plan(Lf, dep, max_row, stream);
        pat_version = version;
        ltb_ready = ub_ready = false;
    }
    if (need_ltb && !ltb_ready) {
        DBuf trp, tci, tsrc, comp;
        transpose_pattern(n, nnzL, Lnat_rp.as<int>(), Lnat_ci.as<int>(), trp, tci, tsrc, stream, tmp);
        comp.alloc(sizeof(int) * (size_t)(nnzL + 1));
        gather_values<int>(tsrc.as<int>(), nat2lev.as<int>(), comp.as<int>(), nnzL, stream);
        build_tri(Ltb, n, nnzL, trp.as<int>(), tci.as<int>(), comp.as<int>(), false, err(), stream, tmp);
        check_err("level schedule");
        ltb_ready = true;
    }
    if (need_ub && !ub_ready) {
        triangle_pattern(n, A_rp.as<int>(), A_ci.as<int>(), false, Unat_rp, Unat_ci, Unat_src, nnzU, stream, tmp);
        build_tri(Ub, n, nnzU, Unat_rp.as<int>(), Unat_ci.as<int>(), Unat_src.as<int>(), false, err(), stream, tmp);
        check_err("level schedule");
        ub_ready = true;
    }
}

void Handle::ensure_work(size_t eb) {
    for (auto &v : vec) v.ensure(eb * (size_t)(n + 1));
}

template <typename T>
void Handle::ensure_scaled() {
    if (dad_valid && dad_version == version) return;
    dscale.ensure(sizeof(T) * (size_t)(n + 1));
    dad.ensure(sizeof(T) * (size_t)(nnz + 1));
    diag_scaling<T>(n, A_rp.as<int>(), A_ci.as<int>(), A_val.as<T>(), nullptr, dscale.as<T>(), nullptr, stream);
    dad_values<T>(n, A_rp.as<int>(), A_ci.as<int>(), A_val.as<T>(), dscale.as<T>(), dad.as<T>(), stream);
    dad_valid = true;
    dad_version = version;
}

template <typename T>
void Handle::ensure_factor(double alpha, bool scaled) {
    ensure_patterns(true, false);
    if (fac_valid && fac_version == version && fac_alpha_req == alpha && fac_scaled == (int)scaled) return;
    fac_valid = false;  // a factorisation that throws leaves no stale factor marked valid
    const T *aval = A_val.as<T>();
    if (scaled) {
        ensure_scaled<T>();
        aval = dad.as<T>();
    }
    // per-entry value arrays carry 16 slots of padding (aligned 16-byte staging in the cluster sweep)
    Lval.ensure(sizeof(T) * (size_t)(nnzL + 16));
    Ltval.ensure(sizeof(T) * (size_t)(nnzL + 16));
    Dvec.ensure(sizeof(T) * (size_t)(n + 1));
    invL.ensure(sizeof(T) * (size_t)(n + 1));
    done_buf.ensure(sizeof(int) * (size_t)(n + 1));
    if (rep_on && !fac_sub_valid) {
        fac_sub_n = own_rows(Lf, rep_src.as<int>(), fac_sub, stream);
        fac_sub_valid = true;
    }
    auto factor_once = [&](double a) {
        gather_values<T>(Lf.psrc.as<int>(), aval, Lval.as<T>(), nnzL, stream);
        timed(PC_FACTOR, 2.0 * (4.0 + sizeof(T)) * nnzL + (double)sizeof(T) * n, [&] {
            ic_factor<T>(Lf, Lval.as<T>(), Dvec.as<T>(), a, err(), ticket() + 2, stream, dep.as<int2>(), max_row,
                         done_buf.as<int>(), fac_backoff_ns, rep_on ? fac_sub.as<int>() : nullptr, fac_sub_n);
            if (rep_on) copy_replica_rows<T>(Lf, rep_src.as<int>(), Lval.as<T>(), Dvec.as<T>(), stream);
        });
        check_err("IC factorisation");
    };
    if (alpha < 0.0) {
        // automatic alpha: MatSolverBase::auto_accel_determine (src/MatSolverBase.cpp:344-391)
        double a = std::fabs(alpha);
        if (a < 0.9 || a > 1.8) a = 1;
        bool ok = false;
        for (int t = 0; t < 80; ++t) {
            factor_once(a);
            all_pivots_positive<T>(n, Dvec.as<T>(), ticket() + 3, stream);
            int flag = 0;
            SSG_CUDA(cudaMemcpyAsync(&flag, ticket() + 3, sizeof(int), cudaMemcpyDeviceToHost, stream));
            SSG_CUDA(cudaStreamSynchronize(stream));
            if (flag) {
                ok = true;
                break;
            }
            a += 0.01;
        }
        if (!ok) {
            a = 1.8;
            factor_once(a);
        }
        alpha_used = a;
    } else {
        factor_once(alpha);
        alpha_used = alpha;
    }
    gather_values<T>(Ltb.psrc.as<int>(), Lval.as<T>(), Ltval.as<T>(), nnzL, stream);
    inv_diag<T>(Lf, Lval.as<T>(), invL.as<T>(), stream);
    invL_lev.ensure(sizeof(T) * (size_t)(n + 1));
    D_lev.ensure(sizeof(T) * (size_t)(n + 1));
    gather_values<T>(Lf.perm.as<int>(), invL.as<T>(), invL_lev.as<T>(), n, stream);
    gather_values<T>(Ltb.perm.as<int>(), Dvec.as<T>(), D_lev.as<T>(), n, stream);
    ++fac_epoch;
    fac_valid = true;
    fac_version = version;
    fac_alpha_req = alpha;
    fac_scaled = (int)scaled;
}

template <typename T>
void Handle::ensure_sgs() {
    ensure_patterns(false, true);
    if (sgs_valid && sgs_version == version) return;
    ensure_scaled<T>();
    Cval.ensure(sizeof(T) * (size_t)(nnzL + 16));
    Uval.ensure(sizeof(T) * (size_t)(nnzU + 16));
    gather_values<T>(Lf.psrc.as<int>(), dad.as<T>(), Cval.as<T>(), nnzL, stream);
    gather_values<T>(Ub.psrc.as<int>(), dad.as<T>(), Uval.as<T>(), nnzU, stream);
    invC.ensure(sizeof(T) * (size_t)(n + 1));
    invU.ensure(sizeof(T) * (size_t)(n + 1));
    inv_diag<T>(Lf, Cval.as<T>(), invC.as<T>(), stream);
    inv_diag<T>(Ub, Uval.as<T>(), invU.as<T>(), stream);
    invC_lev.ensure(sizeof(T) * (size_t)(n + 1));
    invU_lev.ensure(sizeof(T) * (size_t)(n + 1));
    gather_values<T>(Lf.perm.as<int>(), invC.as<T>(), invC_lev.as<T>(), n, stream);
    gather_values<T>(Ub.perm.as<int>(), invU.as<T>(), invU_lev.as<T>(), n, stream);
    sgs_valid = true;
    sgs_version = version;
}

// algorithmic bytes of one sweep: entries (index + value), row pointers, and
// `vecs` streams of n values (rhs, out, aux, D as the mode needs)
static double tri_bytes(const Tri &T, size_t v, int vecs) {
    return (4.0 + (double)v) * T.nnz + 4.0 * (T.n + 1) + (double)vecs * (double)v * T.n;
}

// mean rows per level above which the automatic mode keeps the sync-free sweep
static constexpr double kAutoClusterRowsPerLevel = 4096.0;

bool Handle::cluster_ok(Tri &t, size_t elem, bool ic) {
    if (sweep_mode == 1 || t.n == 0) return false;
    // automatic: one cluster wins while the levels are narrow enough that the
    // per-level latency, not the row count, sets the pace
    if (sweep_mode == 0 && (double)t.n > kAutoClusterRowsPerLevel * (double)t.nlev) return false;
    // the neighbour-synchronised plan (mode 3) serves IC sweeps; a triangle whose plan
    // is infeasible under it falls back to the lockstep plan
    const bool p2p = ic && sweep_mode == 3 && !(t.cl_fail & 2);
    const int ring = p2p ? cl_ring_bytes_p2p : cl_ring_bytes;
    const bool planned = t.cl_ready && t.cl_elem == (int)elem && t.cl_ring_bytes == ring && t.cl_p2p == p2p;
    if (!planned) {
        // a plan of the other kind (or ring) must not be reused
        DBuf tmp;
        t.cl_ready = false;
        if (p2p) {
            cluster_plan(t, elem, ring, stream, tmp, true);
            if (!t.cl_ready) t.cl_fail |= 2;
        }
        if (!t.cl_ready && !(t.cl_fail & 1)) {
            cluster_plan(t, elem, cl_ring_bytes, stream, tmp, false);
            if (!t.cl_ready) t.cl_fail |= 1;
        }
    }
    return t.cl_ready && (ic || !t.cl_p2p);
}

// the push sweep (IC pair, with the reciprocal diagonal): forced by mode 4; the automatic
// choice for real values wherever the one-cluster sweep would be and both push plans fit
bool Handle::push_ok(size_t elem) {
    if (!use_inv_diag || Lf.n == 0) return false;
    if (sweep_mode != 4 && sweep_mode != 0) return false;
    for (const Tri *t : {&Lf, &Ltb})
        if (sweep_mode == 0 &&
            (!push_auto || vtype == SSG_COMPLEX || (double)t->n > kAutoClusterRowsPerLevel * (double)t->nlev))
            return false;
    Tri *pair[2] = {&Lf, &Ltb};
    return push_plan(pair, 2, elem, stream);
}

// z = (L D L^T)^{-1} r using vec[10] as the forward result
template <typename T>
void Handle::apply_precond(const T *d_r, T *d_z, const KState *stp) {
    T *y = vec[10].as<T>();
    const size_t v = sizeof(T);
    if (push_ok(v)) {
        timed(PC_FWD, tri_bytes(Lf, v, 2), [&] {
            sweep_push<T>(Lf, Lval.as<T>(), SW_FWD_DIV, d_r, invL_lev.as<T>(), fac_epoch, y, stp, err(), stream);
        });
        timed(PC_BWD, tri_bytes(Ltb, v, 3), [&] {
            sweep_push<T>(Ltb, Ltval.as<T>(), SW_BWD_IC, y, D_lev.as<T>(), fac_epoch, d_z, stp, err(), stream);
        });
        return;
    }
    if (cluster_ok(Lf, v, true) && cluster_ok(Ltb, v, true)) {
        timed(PC_FWD, tri_bytes(Lf, v, 2), [&] {
            sweep_cluster<T>(Lf, Lval.as<T>(), SW_FWD_DIV, d_r, nullptr, use_inv_diag ? invL_lev.as<T>() : nullptr, y,
                             nullptr, stp, cl_group, err(), stream);
        });
        timed(PC_BWD, tri_bytes(Ltb, v, 3), [&] {
            sweep_cluster<T>(Ltb, Ltval.as<T>(), SW_BWD_IC, nullptr, y, D_lev.as<T>(), d_z, nullptr, stp, cl_group,
                             err(), stream);
        });
        return;
    }
    timed(PC_VEC, (double)v * n, [&] { fill_sentinel_st<T>(y, n, stp, stream); });
    timed(PC_FWD, tri_bytes(Lf, v, 2), [&] {
        sweep_st<T>(Lf, Lval.as<T>(), SW_FWD_DIV, d_r, nullptr, nullptr, y, nullptr, ticket(), err(), stp, stream,
                    swcfg, use_inv_diag ? invL.as<T>() : nullptr);
    });
    timed(PC_VEC, (double)v * n, [&] { fill_sentinel_st<T>(d_z, n, stp, stream); });
    timed(PC_BWD, tri_bytes(Ltb, v, 3), [&] {
        sweep_st<T>(Ltb, Ltval.as<T>(), SW_BWD_IC, nullptr, y, Dvec.as<T>(), d_z, nullptr, ticket() + 1, err(), stp,
                    stream, swcfg, (const T *)nullptr);
    });
}

template <typename T>
static void put_scalar(double *dst, T v);
template <>
void put_scalar<double>(double *dst, double v) {
    dst[0] = v;
    dst[1] = 0.0;
}
template <>
void put_scalar<cplx>(double *dst, cplx v) {
    dst[0] = v.x;
    dst[1] = v.y;
}

template <typename T>
int Handle::solve(int method, double conv_cri, int max_ite, double normB, const T *d_b, T *d_x) {
    const ssg_options &o = opt;
    const bool sgs = (method == SSG_METHOD_MRTR && o.precondition_type == 1);
    const bool scale = sgs || o.is_diag_scale;
    const bool quirks = o.mrtr_reference_quirks != 0;
    cudaStream_t s = stream;
    iters = 0;
    prof.iter = 0;
    prof.pre = true;
    SSG_CUDA(cudaEventRecord(ev[0], s));
    ensure_work(sizeof(T));
    T *b = vec[0].as<T>(), *r = vec[1].as<T>(), *p = vec[2].as<T>(), *z = vec[3].as<T>();
    T *u = vec[4].as<T>(), *y = vec[5].as<T>(), *v = vec[6].as<T>(), *w = vec[7].as<T>();
    T *t1 = vec[8].as<T>(), *best = vec[9].as<T>();
    T *x = d_x;
    double *scal = dscal();
    // |b| as the pointer overloads compute it (src/MatSolverICCG.cpp:48-54)
    if (normB < 0.0) {
        norm2<T>(n, d_b, scal, part.as<double>(), s);
        SSG_CUDA(cudaMemcpyAsync(h_scal, scal, sizeof(double), cudaMemcpyDeviceToHost, s));
        SSG_CUDA(cudaStreamSynchronize(s));
        normB = n ? h_scal[0] : 0.0;
    }
    SSG_CUDA(cudaMemcpyAsync(b, d_b, sizeof(T) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    const T *aval = A_val.as<T>();
    if (scale) {
        // solve_diag_scale / solve_SGS_main: b~ = D b, |b~| replaces the caller's norm
        ensure_scaled<T>();
        vec_mul<T>(n, b, dscale.as<T>(), s);
        norm2<T>(n, b, scal, part.as<double>(), s);
        SSG_CUDA(cudaMemcpyAsync(h_scal, scal, sizeof(double), cudaMemcpyDeviceToHost, s));
        SSG_CUDA(cudaStreamSynchronize(s));
        normB = n ? h_scal[0] : 0.0;
        if (!o.is_init) vec_div<T>(n, x, dscale.as<T>(), s);
        aval = dad.as<T>();
    }
    if (sgs)
        ensure_sgs<T>();
    else
        ensure_factor<T>(o.accel_factor, scale);
    const int *rp = A_rp.as<int>(), *ci = A_ci.as<int>();

    // ---- initial residual
    const bool zero_start = o.is_init != 0;
    if (zero_start && n) SSG_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * (size_t)n, s));
    // the reference's MRTR subtracts A x only when x is zero (src/MatSolverMRTR_ICver.cpp:213-216);
    // with the quirks off the warm start subtracts A x0 as ICCG does
    bool subtract = !zero_start;
    if (method == SSG_METHOD_MRTR && quirks) subtract = false;
    if (subtract) {
        spmv<T>(n, spmv_lanes(), rp, ci, aval, x, v, s);
        vec_sub<T>(n, b, v, r, s);
    } else if (n) {
        SSG_CUDA(cudaMemcpyAsync(r, b, sizeof(T) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    }
    if (sgs && n) {
        // rd = C^{-1} r (src/MatSolverMRTR_SGSver.cpp:118-132)
        if (cluster_ok(Lf, sizeof(T), true)) {
            sweep_cluster<T>(Lf, Cval.as<T>(), SW_FWD_DIV, r, nullptr, use_inv_diag ? invC_lev.as<T>() : nullptr, t1,
                             nullptr, nullptr, cl_group, err(), s);
        } else {
            fill_sentinel_st<T>(t1, n, nullptr, s);
            sweep_st<T>(Lf, Cval.as<T>(), SW_FWD_DIV, r, nullptr, nullptr, t1, nullptr, ticket(), err(), nullptr, s,
                        swcfg, use_inv_diag ? invC.as<T>() : nullptr);
        }
        std::swap(r, t1);
    }
    norm2<T>(n, r, scal, part.as<double>(), s);
    SSG_CUDA(cudaMemcpyAsync(h_scal, scal, sizeof(double), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaStreamSynchronize(s));
    check_err("initial residual");
    const double pure_normR = n ? h_scal[0] : 0.0;

    // ---- convergence set-up (src/MatSolverICCG.cpp:212-237)
    const bool log_on = o.is_save_residual_log != 0;
    auto finish_scale = [&]() {
        if (scale && n) vec_mul<T>(n, x, dscale.as<T>(), s);
        SSG_CUDA(cudaStreamSynchronize(s));
        prof_flush(0);
    };
    if (log_on) residual_log.clear();
    if (normB <= 1.0e-30 && pure_normR <= 1.0e-20) {
        if (log_on) residual_log.assign(1, 0.0);
        finish_scale();
        return SSG_OK;
    }
    const double abs_conv_cri = (normB * conv_cri * 0.9 < 1.0e-20 ? 1.0e-20 : normB * conv_cri * 0.9);
    const double first_normR = pure_normR / normB;
    if (first_normR < conv_cri * 0.5 || pure_normR < abs_conv_cri * 0.5) {
        finish_scale();
        return SSG_OK;
    }
    double normalizer = normB;
    if (o.conv_normalize_type == 1) normalizer = pure_normR;
    else if (o.conv_normalize_type == 2) normalizer = o.conv_normalize_const;

    logbuf.ensure(sizeof(double) * (size_t)(max_ite + 2));
    // ---- device state
    KState &hs = *h_state;
    memset(&hs, 0, sizeof(KState));
    hs.active = max_ite > 0 ? 1 : 0;
    hs.status = max_ite > 0 ? ST_RUNNING : ST_MAXIT;
    hs.max_ite = max_ite;
    hs.diverge_type = o.diverge_judge_type;
    hs.bad_div_count_thres = o.bad_div_count_thres;
    hs.log_enabled = log_on ? 1 : 0;
    hs.quirks = quirks ? 1 : 0;
    hs.conv_cri = conv_cri;
    hs.abs_conv_cri = abs_conv_cri;
    hs.normalizer = normalizer;
    hs.best = 1.0e+6;
    hs.bad_div_val = o.bad_div_val;
    put_scalar<T>(hs.zeta, Sc<T>::one());
    put_scalar<T>(hs.zeta_old, Sc<T>::one());
    put_scalar<T>(hs.nu, Sc<T>::one());
    KState *st = this->st();
    double *log = logbuf.as<double>();
    h_scal[1] = pure_normR / normalizer;
    SSG_CUDA(cudaMemcpyAsync(st, &hs, sizeof(KState), cudaMemcpyHostToDevice, s));
    SSG_CUDA(cudaMemcpyAsync(log, h_scal + 1, sizeof(double), cudaMemcpyHostToDevice, s));
    if (o.is_save_best) SSG_CUDA(cudaMemsetAsync(best, 0, sizeof(T) * (size_t)n, s));

    // ---- method-specific set-up before the loop
    if (method == SSG_METHOD_ICCG) {
        apply_precond<T>(r, z, nullptr);
        SSG_CUDA(cudaMemcpyAsync(p, z, sizeof(T) * (size_t)n, cudaMemcpyDeviceToDevice, s));
        dot_into<T>(n, r, z, st->rur0, part.as<double>(), s);
    } else if (!sgs) {
        apply_precond<T>(r, u, nullptr);
        vec_neg<T>(n, r, y, s);
        apply_precond<T>(y, z, nullptr);
        SSG_CUDA(cudaMemsetAsync(p, 0, sizeof(T) * (size_t)n, s));
        if (zero_start) SSG_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * (size_t)n, s));
    } else {
        vec_neg<T>(n, r, y, s);
        SSG_CUDA(cudaMemsetAsync(p, 0, sizeof(T) * (size_t)n, s));
    }
    SSG_CUDA(cudaEventRecord(ev[1], s));

    // ---- iterations, queued in chunks; every kernel is a no-op once inactive
    const size_t vb = sizeof(T);
    const double nv = (double)vb * n;
    const double spmv_bytes = (4.0 + vb) * nnz + 4.0 * (n + 1) + 2.0 * nv;
    int iter_no = 0;
    const bool sgs_cluster = sgs && cluster_ok(Ub, sizeof(T), false) && cluster_ok(Lf, sizeof(T), false);
    auto one_iteration = [&]() {
        prof.iter = ++iter_no;
        prof.pre = true;
        if (method == SSG_METHOD_ICCG) {
            timed(PC_SPMV, spmv_bytes, [&] { k_spmv_launch<T>(n, spmv_lanes(), rp, ci, aval, p, v, st, true, part.as<double>(), s); });
            timed(PC_VEC, 6 * nv, [&] { iccg_update<T>(n, st, x, r, p, v, part.as<double>(), log, s); });
            prof.pre = false;
            if (o.is_save_best) timed(PC_VEC, 2 * nv, [&] { copy_if_improved<T>(n, st, x, best, s); });
            apply_precond<T>(r, z, st);
            timed(PC_VEC, 2 * nv, [&] { iccg_beta<T>(n, st, r, z, part.as<double>(), s); });
            timed(PC_VEC, 3 * nv, [&] { iccg_p<T>(n, st, p, z, s); });
        } else if (!sgs) {
            timed(PC_SPMV, spmv_bytes, [&] { k_spmv_launch<T>(n, spmv_lanes(), rp, ci, aval, u, v, st, false, part.as<double>(), s); });
            apply_precond<T>(v, w, st);
            timed(PC_VEC, 4 * nv, [&] { mrtr_dots<T>(n, st, w, r, v, y, part.as<double>(), s); });
            timed(PC_VEC, 10 * nv,
                  [&] { mrtr_update<T>(n, st, p, u, x, y, v, r, part.as<double>(), log, quirks, s); });
            prof.pre = false;
            if (o.is_save_best) timed(PC_VEC, 2 * nv, [&] { copy_if_improved<T>(n, st, x, best, s); });
            timed(PC_VEC, 5 * nv, [&] { mrtr_zu<T>(n, st, z, w, u, s); });
        } else {
            // u = U^{-1} rd ; ARd = u + C^{-1}(rd - u)  (src/MatSolverMRTR_SGSver.cpp:184-189)
            if (sgs_cluster) {
                timed(PC_BWD, tri_bytes(Ub, vb, 2), [&] {
                    sweep_cluster<T>(Ub, Uval.as<T>(), SW_BWD_DIV, r, nullptr,
                                     use_inv_diag ? invU_lev.as<T>() : nullptr, u, nullptr, st, cl_group, err(), s);
                });
                timed(PC_FWD, tri_bytes(Lf, vb, 4), [&] {
                    sweep_cluster<T>(Lf, Cval.as<T>(), SW_FWD_EIS, r, u, use_inv_diag ? invC_lev.as<T>() : nullptr,
                                     t1, w, st, cl_group, err(), s);
                });
            } else {
                timed(PC_VEC, nv, [&] { fill_sentinel_st<T>(u, n, st, s); });
                timed(PC_BWD, tri_bytes(Ub, vb, 2), [&] {
                    sweep_st<T>(Ub, Uval.as<T>(), SW_BWD_DIV, r, nullptr, nullptr, u, nullptr, ticket(), err(), st, s,
                                swcfg, use_inv_diag ? invU.as<T>() : nullptr);
                });
                timed(PC_VEC, nv, [&] { fill_sentinel_st<T>(t1, n, st, s); });
                timed(PC_FWD, tri_bytes(Lf, vb, 4), [&] {
                    sweep_st<T>(Lf, Cval.as<T>(), SW_FWD_EIS, r, u, nullptr, t1, w, ticket() + 1, err(), st, s, swcfg,
                                use_inv_diag ? invC.as<T>() : nullptr);
                });
            }
            timed(PC_VEC, 3 * nv, [&] { mrtr_dots<T>(n, st, w, r, w, y, part.as<double>(), s); });
            timed(PC_VEC, 10 * nv, [&] { mrtr_update<T>(n, st, p, u, x, y, w, r, part.as<double>(), log, false, s); });
            prof.pre = false;
            if (o.is_save_best) timed(PC_VEC, 2 * nv, [&] { copy_if_improved<T>(n, st, x, best, s); });
        }
    };
    int chunk = 2;
    int queued = 0;
    for (;;) {
        const int todo = std::min(chunk, max_ite - queued);
        for (int c = 0; c < todo; ++c) one_iteration();
        queued += todo;
        SSG_CUDA(cudaMemcpyAsync(h_state, st, sizeof(KState), cudaMemcpyDeviceToHost, s));
        SSG_CUDA(cudaStreamSynchronize(s));
        if (!h_state->active || queued >= max_ite) break;
        chunk = std::min(chunk * 2, 32);
    }
    SSG_CUDA(cudaEventRecord(ev[2], s));
    check_err("iterations");
    iters = h_state->it;
    prof_flush(iters);
    prof.iter = 0;
    const bool converged = h_state->status == ST_CONVERGED;
    if (log_on) {
        residual_log.resize((size_t)iters + 1);
        SSG_CUDA(cudaMemcpyAsync(residual_log.data(), log, sizeof(double) * ((size_t)iters + 1), cudaMemcpyDeviceToHost,
                                 s));
    }
    if (!converged && o.is_save_best && n)
        SSG_CUDA(cudaMemcpyAsync(x, best, sizeof(T) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    finish_scale();
    float ms0 = 0.f, ms1 = 0.f;
    cudaEventElapsedTime(&ms0, ev[0], ev[1]);
    cudaEventElapsedTime(&ms1, ev[1], ev[2]);
    t_setup_ms = ms0;
    t_iter_ms = ms1;
    return converged ? SSG_OK : SSG_NOT_CONVERGED;
}

// Candidates differ only in schedule (which threads do which rows, and how they
// wait): the sweep mode, the CTAs per SM of the sync-free sweep and, unless
// keep_group, the lanes per row (a different lane count sums a row's entries in
// a different order, so results change at rounding level). Each candidate is
// run once to build its plans, then timed over three applications (median).
template <typename T>
Handle::TuneChoice Handle::autotune(bool keep_group, bool with_push) {
    if (vtype < 0) throw Error{SSG_ERR_STATE, "no matrix set"};
    if (n == 0) return TuneChoice{sweep_mode, swcfg.group, swcfg.cta_per_sm, 0.0};
    ensure_factor<T>(opt.accel_factor, opt.is_diag_scale != 0);
    ensure_work(sizeof(T));
    T *r = vec[1].as<T>(), *z = vec[3].as<T>();
    {
        std::vector<T> ones((size_t)n, Sc<T>::one());
        SSG_CUDA(cudaMemcpyAsync(r, ones.data(), sizeof(T) * (size_t)n, cudaMemcpyHostToDevice, stream));
        SSG_CUDA(cudaStreamSynchronize(stream));
    }
    const int g0 = cl_group;
    std::vector<TuneChoice> cand;
    const std::vector<int> groups = keep_group ? std::vector<int>{g0} : std::vector<int>{4, 8, 16};
    for (int g : groups)
        for (int cps : {0, 2, 4, 8, 16}) cand.push_back({1, g, cps, 0.0});
    for (int g : groups)
        if (g == 4 || g == 8) {
            cand.push_back({2, g, 0, 0.0});
            cand.push_back({3, g, 0, 0.0});
        }
    // the push sweep sums each row in dependency-level order, not by lanes: a candidate
    // only when the summation order is free to change
    if (!keep_group && with_push) cand.push_back({4, 1, 0, 0.0});
    const TuneChoice before{sweep_mode, swcfg.group, swcfg.cta_per_sm, 0.0};
    const int cl_before = cl_group;
    const bool prof_on = prof.on;
    prof.on = false;
    // a batch's sweeps skip ended instances: time every row
    const int *row_inst = swcfg.row_inst;
    swcfg.row_inst = nullptr;
    TuneChoice best{-1, 0, 0, 1e300};
    auto restore = [&](const TuneChoice &k, int clg) {
        prof.on = prof_on;
        swcfg.row_inst = row_inst;
        sweep_mode = k.mode;
        swcfg.group = k.group;
        swcfg.cta_per_sm = k.cta_per_sm;
        cl_group = clg;
    };
    try {
        for (TuneChoice &c : cand) {
            sweep_mode = c.mode;
            swcfg.group = c.group;
            cl_group = c.group;
            swcfg.cta_per_sm = c.cta_per_sm;
            // a cluster candidate whose plan does not fit would time the sync-free sweep again
            if (c.mode == 4 && !push_ok(sizeof(T))) continue;
            if ((c.mode == 2 || c.mode == 3) && !(cluster_ok(Lf, sizeof(T), true) && cluster_ok(Ltb, sizeof(T), true)))
                continue;
            if (c.mode == 3 && !(Lf.cl_p2p && Ltb.cl_p2p)) continue;
            apply_precond<T>(r, z, nullptr);
            check_err("autotune");
            float t[3];
            for (float &ti : t) {
                SSG_CUDA(cudaEventRecord(ev[0], stream));
                apply_precond<T>(r, z, nullptr);
                SSG_CUDA(cudaEventRecord(ev[1], stream));
                SSG_CUDA(cudaEventSynchronize(ev[1]));
                SSG_CUDA(cudaEventElapsedTime(&ti, ev[0], ev[1]));
            }
            check_err("autotune");
            std::sort(t, t + 3);
            c.ms = t[1];
            if (c.ms < best.ms) best = c;
        }
    } catch (...) {
        restore(before, cl_before);
        throw;
    }
    if (best.mode < 0) {
        restore(before, cl_before);
        throw Error{SSG_ERR_STATE, "autotune: no candidate ran"};
    }
    restore(best, best.group);
    return best;
}

template Handle::TuneChoice Handle::autotune<double>(bool, bool);
template Handle::TuneChoice Handle::autotune<cplx>(bool, bool);
template int Handle::solve<double>(int, double, int, double, const double *, double *);
template int Handle::solve<cplx>(int, double, int, double, const cplx *, cplx *);
template void Handle::ensure_factor<double>(double, bool);
template void Handle::ensure_factor<cplx>(double, bool);
template void Handle::apply_precond<double>(const double *, double *, const KState *);
template void Handle::apply_precond<cplx>(const cplx *, cplx *, const KState *);

}  // namespace ssg
