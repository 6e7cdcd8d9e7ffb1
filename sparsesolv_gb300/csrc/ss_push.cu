// ss_push.cu -- one-cluster push sweeps for the IC pair (forward L y = r with
// 1/L_ii, backward x = y - D L^T x), the triangular solves of
// MatSolverBase::IC_frbc_process (src/MatSolverBase.cpp:177-231).
//
// The level-synchronous cluster sweep (ss_cluster.cu) pays, at every one of the
// ~1,400 dependency levels of an 80^3 system, a cluster barrier, the loads of
// the rows' dependencies from other CTAs' shared memory, and the row sums on
// GB300's narrow FP64 pipe, one after another: 2.6 us per level. Here no
// barrier spans the cluster:
//
//   * every CTA owns a contiguous chunk of each level (the lockstep plan's
//     partition) and keeps the values it produced in a shared-memory ring;
//   * a finished value is pushed into the shared memory of every CTA that
//     reads it (st.async), each push counted on the receiver's mbarrier for the
//     producer's level, so a CTA starts level l as soon as its own level l-1 is
//     done and the values other CTAs produced at level l-1 have landed;
//   * each row's entries are summed in the order of their dependency levels,
//     oldest first. One warp group sums the entries of levels <= l-1 of level
//     l+1's rows while the other finishes level l (its entries of level l-1,
//     one fused multiply-add each after the wait) and pushes the results;
//   * rows fill warps densely: a warp instruction on GB300's FP64 pipe costs
//     the same with 17 or 32 active lanes;
//   * each level's chunk is one record (ss_push_plan.hpp) staged by one
//     cp.async.bulk copy NB - 1 levels ahead;
//   * a CTA runs at most LEAD levels ahead of the slowest CTA (progress words
//     polled through distributed shared memory, rarely binding), which bounds
//     how long a receive slot or a receive barrier phase must stay valid; the
//     plan proves every slot reuse safe under that bound or is infeasible.
//
// Per-row arithmetic: the older entries go into two interleaved partial sums
// (the forward right-hand side starts the first), which are added and scaled
// (forward: by 1/L_ii; backward: aux + D * sum); each newest entry adds
// -(v * 1/L_ii) * x (forward) or -(v * D) * x (backward) with a fused
// multiply-add. The summation order differs from the other sweeps', so results
// agree with theirs at rounding level; the push sweep is deterministic run to
// run.
//
// Every wait is bounded (the handle's spin limit); on a timeout the kernel
// records ERR_TIMEOUT, every CTA leaves its level loop at the next step, waits
// for the copies it issued and for the pushes in flight, and returns.
#include <algorithm>
#include <exception>
#include <thread>

#include "sparsesolv_gb300.h"
#include "ss_internal.cuh"
#include "ss_krylov.cuh"

namespace ssg {

// ---------------------------------------------------------------- device helpers
__device__ __forceinline__ unsigned ps_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned ps_mapa(unsigned local_addr, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local_addr), "r"(rank));
    return r;
}
__device__ __forceinline__ void ps_mbar_init(unsigned a, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void ps_mbar_expect(unsigned a, unsigned tx) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(tx) : "memory");
}
// the phase with this parity has completed (a non-blocking test). Acquire at
// cluster scope: values other CTAs pushed with st.async are visible.
__device__ __forceinline__ bool ps_mbar_test(unsigned a, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
// the same at CTA scope (bulk copies into this CTA's shared memory)
__device__ __forceinline__ bool ps_mbar_test_cta(unsigned a, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void ps_fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void ps_bulk_g2s(unsigned dst, const void *src, unsigned bytes, unsigned mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}
__device__ __forceinline__ void ps_cp16(unsigned dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void ps_cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void ps_cp_wait3() { asm volatile("cp.async.wait_group 3;" ::: "memory"); }
__device__ __forceinline__ void ps_cp_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void ps_st_release(unsigned a, unsigned v) {
    asm volatile("st.release.cluster.shared::cta.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ps_ld_acquire(unsigned cluster_addr) {
    unsigned v;
    asm volatile("ld.acquire.cluster.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(cluster_addr) : "memory");
    return v;
}
__device__ __forceinline__ void ps_cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// value pushed into another CTA's shared memory, counted on its mbarrier
__device__ __forceinline__ void ps_push(unsigned raddr, double v, unsigned rmbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];" ::"r"(raddr),
                 "l"((unsigned long long)__double_as_longlong(v)), "r"(rmbar)
                 : "memory");
}
__device__ __forceinline__ void ps_push(unsigned raddr, float v, unsigned rmbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];" ::"r"(raddr),
                 "r"(__float_as_uint(v)), "r"(rmbar)
                 : "memory");
}
__device__ __forceinline__ void ps_push(unsigned raddr, cplx v, unsigned rmbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.b64 [%0], {%1, %2}, [%3];" ::"r"(raddr),
                 "l"((unsigned long long)__double_as_longlong(v.x)),
                 "l"((unsigned long long)__double_as_longlong(v.y)), "r"(rmbar)
                 : "memory");
}
__device__ __forceinline__ void ps_push(unsigned raddr, cplxf v, unsigned rmbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.b32 [%0], {%1, %2}, [%3];" ::"r"(raddr),
                 "r"(__float_as_uint(v.x)), "r"(__float_as_uint(v.y)), "r"(rmbar)
                 : "memory");
}

template <typename T>
__device__ __forceinline__ T ps_ldg(const T *p) {
    return __ldcg(p);
}
template <>
__device__ __forceinline__ cplx ps_ldg<cplx>(const cplx *p) {
    const double2 v = __ldcg((const double2 *)p);
    return {v.x, v.y};
}
template <>
__device__ __forceinline__ cplxf ps_ldg<cplxf>(const cplxf *p) {
    const float2 v = __ldcg((const float2 *)p);
    return {v.x, v.y};
}

struct PsArgs {
    int nlev;
    const int4 *tab;  // per (level, CTA): {record offset / 16, record bytes / 16, bytes pushed here, 0}
    const unsigned char *rec;
    void *out;
    const KState *st;
    int *err;
    PushLayout L;
};

template <typename T, int MODE>
__global__ void __launch_bounds__(PS_THREADS, 1) k_sweep_push(PsArgs a) {
    if (a.st && !a.st->active) return;  // uniform across the cluster
    extern __shared__ __align__(16) unsigned char ps_smem[];
    const PushLayout &L = a.L;
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(ps_smem);
    T *X = (T *)(ps_smem + L.o_x);  // own ring [S_own], then receive ring [S_recv]
    const unsigned mbr = sbase + L.o_mbr, mbs = sbase + L.o_mbs, prog = sbase + L.o_prog;
    const int4 *tabring = (const int4 *)(ps_smem + L.o_tabring);  // [0, 4): staging, [4, 8): arming
    const int rank = (int)ps_rank();
    const int C = (int)gridDim.x;
    const int tid = threadIdx.x;
    const bool stager = tid >= 2 * PS_CT;
    const bool newg = tid < PS_CT;  // newest-entry group; [PS_CT, 2 PS_CT): older-entry group
    const int ct = tid & (PS_CT - 1);
    const int lane = tid & 31;
    const int nlev = a.nlev;
    const int4 *tab = a.tab;
    T *out = (T *)a.out;
    T *hand = (T *)(ps_smem + L.o_base);  // [level parity][PS_MAXQ * PS_CT] partial sums, by row
    const unsigned long long lim = spin_limit_ns(a.err);
    constexpr int VB = (int)sizeof(T);
    const int bufb = ps_al16(L.cap_rec);

    // stage level l's record into buffer l % NB: one bulk copy
    auto stage = [&](int l, int4 e) {
        const int b = l % L.NB;
        const unsigned mb = mbs + 8u * b;
        ps_mbar_expect(mb, 16u * (unsigned)e.y);
        ps_bulk_g2s(sbase + L.o_buf + b * bufb, a.rec + 16ll * e.x, 16u * (unsigned)e.y, mb);
    };
    // what step s needs, into ring slot s % 4 (one commit group per step): the table entry
    // of the level it stages (s + NB - 1, lane 0) and of the level whose receive phase it
    // arms (s - 2 + R, lane 1)
    auto prefetch_step = [&](int s) {
        const int ls = s + L.NB - 1, la = s - 2 + L.R;
        if (lane == 0 && ls < nlev) ps_cp16(sbase + L.o_tabring + 16u * (s & 3), tab + (size_t)ls * C + rank);
        if (lane == 1 && s >= 2 && la < nlev)
            ps_cp16(sbase + L.o_tabring + 64u + 16u * (s & 3), tab + (size_t)la * C + rank);
        ps_cp_commit();
    };
    // bounded wait for a barrier phase; false on a timeout or another CTA's error
    auto wait_phase = [&](unsigned bar, unsigned parity, bool cluster) -> bool {
        auto test = [&]() { return cluster ? ps_mbar_test(bar, parity) : ps_mbar_test_cta(bar, parity); };
        if (test()) return true;
        const unsigned long long t0 = gtimer();
        int polls = 0;
        while (!test()) {
            if ((++polls & 63) == 0) {
                if (*(volatile int *)a.err) return false;
                if (gtimer() - t0 > lim) {
                    atomicExch(a.err, ERR_TIMEOUT);
                    return false;
                }
            }
        }
        return true;
    };

    // ---- set-up: barriers, progress word, the first staged levels, the first receive phases
    if (tid == 2 * PS_CT) {
        for (int i = 0; i < L.R; ++i) ps_mbar_init(mbr + 8u * i, 1);
        for (int i = 0; i < L.NB; ++i) ps_mbar_init(mbs + 8u * i, 1);
        *(volatile unsigned *)(ps_smem + L.o_prog) = 0u;
        ps_fence_mbar_init();
    }
    __syncthreads();
    if (stager) {
        if (lane == 0) {
            // receive phases of producer levels 0..R-1: the bytes other CTAs push here at each
            for (int l = 0; l < L.R && l < nlev; ++l) ps_mbar_expect(mbr + 8u * l, (unsigned)tab[(size_t)l * C + rank].z);
            for (int l = 0; l < L.NB - 1 && l < nlev; ++l) stage(l, tab[(size_t)l * C + rank]);
        }
        __syncwarp();
        for (int q = 0; q < 4; ++q) prefetch_step(q);  // what steps 0..3 need
    }
    // no CTA pushes before every CTA's barriers are initialised and armed
    ps_cluster_sync();

    bool bad = false;
    int seen = 0;      // stager lane q: the last progress seen of CTA q
    int produced = 0;  // values this CTA has produced (own ring position)
    // Older entries of level l's rows, by the older-entry group during step l-1 (the
    // entries of levels <= l-2), scaled so that each newest entry is one fused
    // multiply-add after the wait; the newest values are rescaled in place in the
    // staged record.
    auto old_part = [&](int l) {
        const int b = l % L.NB;
        if (!wait_phase(mbs + 8u * b, (unsigned)((l / L.NB) & 1), false)) {
            bad = true;
            return;
        }
        unsigned char *rb = ps_smem + L.o_buf + b * bufb;
        const int *hd = (const int *)rb;
        const int cnt = hd[0];
        const bool hasg = (hd[3] >> 16) != 0;
        const PsRec R = ps_rec(cnt, hd[1], hd[2], VB);
        const int4 *info = (const int4 *)(rb + R.o_info);
        const int *code = (const int *)(rb + R.o_code);
        const T *val = (const T *)(rb + R.o_val);
        const T *lv = (const T *)(rb + R.o_lv);
        const T *rhs = (const T *)(rb + R.o_rhs);
        T *hb = hand + (l & 1) * (PS_MAXQ * PS_CT);
#pragma unroll
        for (int j = 0; j < PS_MAXQ; ++j) {
            const int p = j * PS_CT + ct;
            if (p >= cnt) continue;
            const int4 ri = info[p];
            if (ri.z < 0) continue;
            const int e = ri.x, nold = ri.y & 0xFFFF;
            T s0 = (MODE == SW_FWD_DIV) ? rhs[p] : Sc<T>::zero(), s1 = Sc<T>::zero();
            int k = 0;
            if (!hasg) {
                // every read from shared memory: no branch, the loads run ahead of the sums
#pragma unroll 2
                for (; k + 2 <= nold; k += 2) {
                    const int i0 = e + 32 * k;
                    s0 = madd(s0, -val[i0], X[-1 - code[i0]]);
                    s1 = madd(s1, -val[i0 + 32], X[-1 - code[i0 + 32]]);
                }
                if (k < nold) {
                    const int i = e + 32 * k;
                    s0 = madd(s0, -val[i], X[-1 - code[i]]);
                }
            } else {
                for (; k + 2 <= nold; k += 2) {
                    const int i0 = e + 32 * k;
                    const int c0 = code[i0], c1 = code[i0 + 32];
                    const T x0 = c0 < 0 ? X[-1 - c0] : ps_ldg(out + c0);
                    const T x1 = c1 < 0 ? X[-1 - c1] : ps_ldg(out + c1);
                    s0 = madd(s0, -val[i0], x0);
                    s1 = madd(s1, -val[i0 + 32], x1);
                }
                if (k < nold) {
                    const int i = e + 32 * k, c = code[i];
                    s0 = madd(s0, -val[i], c < 0 ? X[-1 - c] : ps_ldg(out + c));
                }
            }
            const T sum = s0 + s1;
            const T d = lv[p];
            hb[p] = (MODE == SW_FWD_DIV) ? sum * d : madd(rhs[p], d, sum);
        }
    };

    if (!newg && !stager && nlev > 0) old_part(0);

    int l = 0;
    for (; l < nlev; ++l) {
        // step l: every thread has finished step l-1 (own values of level l-1 are in X, the
        // partial sums of level l are handed over)
        if (__syncthreads_or(bad)) break;
        if (stager) {
            // this step's table entries landed (prefetched four steps ago)
            ps_cp_wait3();
            __syncwarp();
            if (lane == 0) {
                // re-arm the receive phase of producer level l-2 for producer level l-2+R: every
                // thread of this CTA has passed its wait on level l-2 (done at step l-1)
                if (l >= 2 && l - 2 + L.R < nlev) ps_mbar_expect(mbr + 8u * ((l - 2) % L.R), (unsigned)tabring[4 + (l & 3)].z);
                // steps before l are complete; published every 4 steps (the others rely on a
                // lower bound of this CTA's progress only)
                if ((l & 3) == 0) ps_st_release(prog, (unsigned)l);
                if (l + L.NB - 1 < nlev) stage(l + L.NB - 1, tabring[l & 3]);
            }
            __syncwarp();
            prefetch_step(l + 4);
            // before step l+1: no CTA more than LEAD levels behind (lane q watches CTA q)
            const int need = l + 1 - L.LEAD;
            if (need > seen && lane < C && lane != rank) {
                const unsigned ra = ps_mapa(prog, (unsigned)lane);
                if ((seen = (int)ps_ld_acquire(ra)) < need) {
                    const unsigned long long t0 = gtimer();
                    int polls = 0;
                    while ((seen = (int)ps_ld_acquire(ra)) < need) {
                        __nanosleep(64);  // a slower CTA's shared memory serves its own work first
                        if ((++polls & 63) == 0) {
                            if (*(volatile int *)a.err) {
                                bad = true;
                                break;
                            }
                            if (gtimer() - t0 > lim) {
                                atomicExch(a.err, ERR_TIMEOUT);
                                bad = true;
                                break;
                            }
                        }
                    }
                }
            }
            continue;
        }
        // values other CTAs produced at level l-1 have landed (both groups read them)
        if (l >= 1 && !wait_phase(mbr + 8u * ((l - 1) % L.R), (unsigned)(((l - 1) / L.R) & 1), true)) {
            bad = true;
            continue;
        }
        if (!newg) {
            if (l + 1 < nlev) old_part(l + 1);
            continue;
        }
        const int b = l % L.NB;
        const unsigned char *rb = ps_smem + L.o_buf + b * bufb;
        const int *hd = (const int *)rb;
        const int cnt = hd[0];
        const PsRec R = ps_rec(cnt, hd[1], hd[2], VB);
        const int4 *info = (const int4 *)(rb + R.o_info);
        const int *code = (const int *)(rb + R.o_code);
        const int *push = (const int *)(rb + R.o_push);
        const T *val = (const T *)(rb + R.o_val);
        const T *hb = hand + (l & 1) * (PS_MAXQ * PS_CT);
        const unsigned bar_l = mbr + 8u * (l % L.R);
#pragma unroll
        for (int j = 0; j < PS_MAXQ; ++j) {
            const int p = j * PS_CT + ct;
            if (p >= cnt) continue;
            const int4 ri = info[p];
            if (ri.z < 0) continue;
            const int e = ri.x, nold = ri.y & 0xFFFF, len = ri.y >> 16;
            T res = hb[p];
            // the newest entries always come from shared memory (the plan guarantees it)
            for (int k = nold; k < len; ++k) {
                const int i = e + 32 * k;
                res = madd(res, val[i], X[-1 - code[i]]);
            }
            X[(produced + p) % L.S_own] = res;
            const int pe = info[p + 1].w;
            for (int k = ri.w; k < pe; ++k) {
                const int pk = push[k];
                const unsigned c = (unsigned)pk >> 24, slot = (unsigned)pk & 0xFFFFFFu;
                ps_push(ps_mapa(sbase + L.o_x + (unsigned)VB * (unsigned)(L.S_own + slot), c), res, ps_mapa(bar_l, c));
            }
            out[ri.z] = res;
        }
        produced += cnt;
    }
    // ---- leave: uniform per CTA (the loop ends for all its threads at the same step)
    __syncthreads();
    const bool failed = l < nlev;
    if (stager) {
        ps_cp_wait0();
        if (failed && lane == 0) {
            // bulk copies issued for levels not consumed: wait for them (bounded) before the
            // shared memory goes away
            for (int lv = l; lv < l + L.NB - 1 && lv < nlev; ++lv) {
                const int b = lv % L.NB;
                const unsigned long long t0 = gtimer();
                while (!ps_mbar_test_cta(mbs + 8u * b, (unsigned)((lv / L.NB) & 1)) && gtimer() - t0 < 1000000ull) {
                }
            }
        }
    }
    // no CTA leaves while another may still read its progress word or push into it
    ps_cluster_sync();
    if (failed) {
        // a failed run may leave pushes issued before the failure in flight: let them land
        const unsigned long long t0 = gtimer();
        while (gtimer() - t0 < 20000ull) {
        }
    }
}

// ---------------------------------------------------------------- record values (per factor, per sweep)
// the factor's values and per-row vector into the records: rec[dval[k]] = val[vmap[k]], rec[dlv[t]] = lvec[t]
template <typename T>
__global__ void k_push_fill(int nent, int n, const int *vmap, const int *dval, const int *dlv, const T *val,
                            const T *lvec, T *rec) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nent) rec[dval[k]] = val[vmap[k]];
    if (k < n) rec[dlv[k]] = lvec[k];
}
// the newest entries pre-scaled by their row's 1/L_ii (forward) or D (backward), once per factor,
// so that each is one fused multiply-add in the sweep: rec[dval[k]] = -(val[vmap[k]] * lvec[t])
template <typename T>
__global__ void k_push_scale_newest(int nnew, const int2 *dnew, const int *vmap, const int *dval, const T *val,
                                    const T *lvec, T *rec) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nnew) return;
    const int2 kt = dnew[q];
    rec[dval[kt.x]] = -(val[vmap[kt.x]] * lvec[kt.y]);
}
// the right-hand side of one sweep into the records, by level-ordered row: rec[drhs[t]] = v[perm[t]]
template <typename T>
__global__ void k_push_rhs(int n, const int *perm, const int *drhs, const T *v, T *rec) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) rec[drhs[t]] = v[perm[t]];
}

static int g_push_cluster = -1;

static int push_cluster_size() {
    if (g_push_cluster >= 0) return g_push_cluster;
    g_push_cluster = 0;
    auto kern = k_sweep_push<double, SW_FWD_DIV>;
    for (int C : {16, 8}) {
        if (C > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
            (void)cudaGetLastError();
            continue;
        }
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, PS_SMEM_MAX) != cudaSuccess) {
            (void)cudaGetLastError();
            break;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(C);
        cfg.blockDim = dim3(PS_THREADS);
        cfg.dynamicSmemBytes = PS_SMEM_MAX;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = C;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess && nclusters > 0) {
            g_push_cluster = C;
            break;
        }
        (void)cudaGetLastError();
    }
    return g_push_cluster;
}

template <typename I>
static void upload(DBuf &d, const std::vector<I> &h, size_t pad_elems, cudaStream_t s) {
    d.ensure(sizeof(I) * (h.size() + pad_elems));
    SSG_CUDA(cudaMemsetAsync(d.p, 0, sizeof(I) * (h.size() + pad_elems), s));
    if (!h.empty()) SSG_CUDA(cudaMemcpyAsync(d.p, h.data(), sizeof(I) * h.size(), cudaMemcpyHostToDevice, s));
}

// The plans: once per pattern and value size, on the host (ss_push_plan.cpp). The triangles
// of one call (the IC pair) are planned side by side on host threads; each plan depends on
// its own triangle only, so the result is the one a call per triangle gives.
bool push_plan(Tri *const *tris, int count, size_t elem_bytes, cudaStream_t s) {
    const int elem = (int)elem_bytes;
    const int ebit = elem == 4 ? 1 : elem == 8 ? 2 : 4;
    const int slot = elem == 4 ? 0 : elem == 8 ? 1 : 2;
    struct Job {
        Tri *T;
        std::vector<int> prp, pci, perm, level, ipos;
        PushPlanHost H;
    };
    std::vector<Job> jobs;
    const int C = push_cluster_size();
    for (int i = 0; i < count; ++i) {
        Tri &T = *tris[i];
        PushPlan &P = T.push[slot];
        if (P.n != T.n || P.nnz != T.nnz || P.nlev != T.nlev) {
            // made for another triangle: start over (the shape is recorded before any attempt,
            // so an infeasible plan is not retried on every call)
            P.ready = false;
            P.fail = 0;
            P.n = T.n;
            P.nnz = T.nnz;
            P.nlev = T.nlev;
        }
        if (P.ready && P.elem == elem) continue;
        if (P.fail & ebit) return false;
        P.ready = false;
        if (C <= 0 || T.n == 0 || T.nlev < 2) {
            P.fail |= ebit;
            return false;
        }
        jobs.push_back(Job{&T, {}, {}, {}, {}, {}, {}});
    }
    if (jobs.empty()) return true;
    for (Job &j : jobs) {
        const Tri &T = *j.T;
        const int n = T.n;
        j.prp.resize(n + 1);
        j.pci.resize(T.nnz);
        j.perm.resize(n);
        j.level.resize(n);
        j.ipos.resize(n);
        SSG_CUDA(cudaMemcpyAsync(j.prp.data(), T.prp.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
        SSG_CUDA(cudaMemcpyAsync(j.pci.data(), T.pci.p, sizeof(int) * (size_t)T.nnz, cudaMemcpyDeviceToHost, s));
        SSG_CUDA(cudaMemcpyAsync(j.perm.data(), T.perm.p, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
        SSG_CUDA(cudaMemcpyAsync(j.level.data(), T.level.p, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
        SSG_CUDA(cudaMemcpyAsync(j.ipos.data(), T.ipos.p, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    }
    SSG_CUDA(cudaStreamSynchronize(s));
    auto plan = [&](Job &j) {
        const Tri &T = *j.T;
        j.H = push_plan_host(T.n, T.nlev, T.lptr.data(), j.prp.data(), j.pci.data(), j.perm.data(), j.level.data(),
                             j.ipos.data(), C, elem);
    };
    {
        std::vector<std::thread> pool;
        std::vector<std::exception_ptr> errs(jobs.size());
        auto run = [&](size_t i) {
            try {
                plan(jobs[i]);
            } catch (...) {
                errs[i] = std::current_exception();
            }
        };
        std::vector<size_t> here{0};  // plans run on this thread (a thread that cannot start)
        for (size_t i = 1; i < jobs.size(); ++i) {
            try {
                pool.emplace_back(run, i);
            } catch (...) {
                here.push_back(i);
            }
        }
        for (size_t i : here) run(i);
        for (auto &t : pool) t.join();
        for (auto &e : errs)
            if (e) std::rethrow_exception(e);
    }
    bool all = true;
    for (Job &j : jobs) {
        PushPlan &P = j.T->push[slot];
        const PushPlanHost &H = j.H;
        if (!H.ok) {
            P.fail |= ebit;
            all = false;
            continue;
        }
        upload(P.tab, H.tab, 4, s);
        upload(P.rec, H.rec, 16, s);
        upload(P.vmap, H.vmap, 4, s);
        upload(P.dval, H.dval, 4, s);
        upload(P.dlv, H.dlv, 4, s);
        upload(P.drhs, H.drhs, 4, s);
        upload(P.perm, j.perm, 4, s);
        upload(P.dnew, H.dnew, 4, s);
        SSG_CUDA(cudaStreamSynchronize(s));
        P.key_val = P.key_lv = nullptr;
        P.key_epoch = ~0ull;
        P.elem = elem;
        P.C = C;
        P.nent = H.nent;
        P.npush = H.npush;
        P.nnew = (int)(H.dnew.size() / 2);
        P.lay = H.lay;
        P.ready = true;
    }
    return all;
}

template <typename T>
void sweep_push(Tri &tri, const T *val, int mode, const T *rhs, const T *lvec, unsigned long long epoch, T *out,
                const KState *st, int *err, cudaStream_t s) {
    PushPlan &P = tri.push[sizeof(T) == 4 ? 0 : sizeof(T) == 8 ? 1 : 2];
    if (tri.n == 0) return;
    if (!P.ready || P.elem != (int)sizeof(T) || P.n != tri.n || P.nnz != tri.nnz || P.nlev != tri.nlev)
        throw Error{SSG_ERR_STATE, "push sweep without a plan for this triangle"};
    T *rec = P.rec.as<T>();
    if (P.key_val != val || P.key_lv != lvec || P.key_epoch != epoch) {
        const int m = std::max(P.nent, tri.n);
        k_push_fill<T><<<div_up(std::max(m, 1), 256), 256, 0, s>>>(P.nent, tri.n, P.vmap.as<int>(), P.dval.as<int>(),
                                                                   P.dlv.as<int>(), val, lvec, rec);
        SSG_LAUNCHED();
        if (P.nnew > 0) {
            k_push_scale_newest<T><<<div_up(P.nnew, 256), 256, 0, s>>>(P.nnew, P.dnew.as<int2>(), P.vmap.as<int>(),
                                                                       P.dval.as<int>(), val, lvec, rec);
            SSG_LAUNCHED();
        }
        P.key_val = val;
        P.key_lv = lvec;
        P.key_epoch = epoch;
    }
    k_push_rhs<T><<<div_up(tri.n, 256), 256, 0, s>>>(tri.n, P.perm.as<int>(), P.drhs.as<int>(), rhs, rec);
    SSG_LAUNCHED();
    PsArgs a;
    a.nlev = tri.nlev;
    a.tab = P.tab.as<int4>();
    a.rec = P.rec.as<unsigned char>();
    a.out = out;
    a.st = st;
    a.err = err;
    a.L = P.lay;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(P.C);
    cfg.blockDim = dim3(PS_THREADS);
    cfg.dynamicSmemBytes = P.lay.total;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = P.C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
#define SSG_PS(M)                                                                                             \
    do {                                                                                                      \
        auto kern = k_sweep_push<T, M>;                                                                       \
        static bool prepared = false;                                                                         \
        if (!prepared) {                                                                                      \
            if (P.C > 8) SSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)); \
            SSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, PS_SMEM_MAX));   \
            prepared = true;                                                                                  \
        }                                                                                                     \
        SSG_CUDA(cudaLaunchKernelEx(&cfg, kern, a));                                                          \
    } while (0)
    if (mode == SW_FWD_DIV) SSG_PS(SW_FWD_DIV);
    else if (mode == SW_BWD_IC) SSG_PS(SW_BWD_IC);
    else throw Error{SSG_ERR_STATE, "push sweep serves the IC pair only"};
#undef SSG_PS
    SSG_LAUNCHED();
}

#define SSG_INST(T)                                                                                             \
    template void sweep_push<T>(Tri &, const T *, int, const T *, const T *, unsigned long long, T *,          \
                                const KState *, int *, cudaStream_t);
SSG_INST(double)
SSG_INST(cplx)
SSG_INST(float)
SSG_INST(cplxf)
#undef SSG_INST

}  // namespace ssg
