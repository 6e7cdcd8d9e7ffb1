// ss_cluster.cu -- level-synchronous triangular sweeps inside one thread-block
// cluster, with recent results exchanged through distributed shared memory.
//
// The sync-free sweep (ss_trsv.cu) pays several L2 round trips per dependency
// level (publish, poll, gather): about 2.8 us per level on GB300. Here one
// cluster of C CTAs (16 where non-portable cluster sizes are allowed, else 8)
// runs the whole sweep, one cluster barrier per level:
//
//   compute warps   solve their share of level l (a contiguous run of the
//                   level-ordered rows), reading each dependency either from
//                   the producing CTA's shared-memory ring (ld.shared::cluster)
//                   or, when it is older than the ring holds, from L2; they
//                   write results only to their own ring, so their
//                   barrier.cluster.arrive.release has no global store to wait for;
//                   then they stage level l+3's matrix span and level l+2's
//                   gathered inputs with cp.async while the barrier completes.
//   store warp      copies level l's results from the ring to the output
//                   vector in HBM; it arrives relaxed, except at every K-th
//                   level, where its release (issued before that level's stores)
//                   publishes everything it stored earlier.
//
// Which source serves each dependency is decided once per pattern (cluster_plan):
// the ring when its slot cannot have been overwritten before the consumer's
// level ends, memory when a release covering the value precedes the
// consumer's level. An entry that satisfies neither makes the plan infeasible
// and the sync-free sweep is used. There is no spin-wait: the only waits are
// cp.async completion, CTA barriers and cluster barriers, reached the same
// number of times by every thread.
#include <algorithm>

#include "sparsesolv_gb300.h"
#include "ss_internal.cuh"
#include "ss_krylov.cuh"

namespace ssg {

constexpr int CL_SLOT_BITS = 20;
constexpr int CL_STORE_K = 8;   // store warp releases every K levels
constexpr int CL_SPAN_BUFS = 5; // matrix span staged 4 levels ahead
constexpr int CL_GATH_BUFS = 3; // gathered inputs staged 2 levels ahead
constexpr int CL_PAD = 4;       // entries copied beyond a span to keep the 16-byte copies aligned
constexpr int CL_LEAD = 4;      // neighbour-synchronised sweep: levels a CTA may run ahead of every other

__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_arrive_release() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_arrive_relaxed() {
    asm volatile("barrier.cluster.arrive.relaxed.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait_acquire() {
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
__device__ __forceinline__ unsigned map_shared(unsigned local_addr, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local_addr), "r"(rank));
    return r;
}
__device__ __forceinline__ void bar_arrive(int id, int count) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_sync(int id, int count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
// progress word of the neighbour-synchronised sweep: levels this CTA has completed
__device__ __forceinline__ void st_release_progress(unsigned local_addr, unsigned v) {
    asm volatile("st.release.cluster.shared::cta.u32 [%0], %1;" ::"r"(local_addr), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_progress(unsigned cluster_addr) {
    unsigned v;
    asm volatile("ld.acquire.cluster.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(cluster_addr) : "memory");
    return v;
}
template <int BYTES>
__device__ __forceinline__ void cp_async(unsigned dst, const void *src) {
    if (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(dst), "l"(src), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev2() { asm volatile("cp.async.wait_group 2;" ::: "memory"); }

template <typename T>
__device__ __forceinline__ T ld_dsmem(unsigned addr);
template <>
__device__ __forceinline__ double ld_dsmem<double>(unsigned addr) {
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr));
    return v;
}
template <>
__device__ __forceinline__ float ld_dsmem<float>(unsigned addr) {
    float v;
    asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}
template <>
__device__ __forceinline__ cplx ld_dsmem<cplx>(unsigned addr) {
    cplx v;
    asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(addr));
    return v;
}
template <>
__device__ __forceinline__ cplxf ld_dsmem<cplxf>(unsigned addr) {
    cplxf v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}
// generic address of the same shared-memory location in CTA `rank` of the cluster
__device__ __forceinline__ unsigned long long mapa_generic(const void *p, unsigned rank) {
    unsigned long long r;
    asm volatile("mapa.u64 %0, %1, %2;" : "=l"(r) : "l"(p), "r"(rank));
    return r;
}
// one load for either a global address or a distributed shared-memory address;
// relaxed at cluster scope, so a global line is never served stale from L1
template <typename T>
__device__ __forceinline__ T ld_rc(unsigned long long a);
template <>
__device__ __forceinline__ double ld_rc<double>(unsigned long long a) {
    double v;
    asm volatile("ld.relaxed.cluster.f64 %0, [%1];" : "=d"(v) : "l"(a) : "memory");
    return v;
}
template <>
__device__ __forceinline__ float ld_rc<float>(unsigned long long a) {
    float v;
    asm volatile("ld.relaxed.cluster.f32 %0, [%1];" : "=f"(v) : "l"(a) : "memory");
    return v;
}
template <>
__device__ __forceinline__ cplx ld_rc<cplx>(unsigned long long a) {
    cplx v;
    asm volatile("ld.relaxed.cluster.f64 %0, [%1];" : "=d"(v.x) : "l"(a) : "memory");
    asm volatile("ld.relaxed.cluster.f64 %0, [%1];" : "=d"(v.y) : "l"(a + 8) : "memory");
    return v;
}
template <>
__device__ __forceinline__ cplxf ld_rc<cplxf>(unsigned long long a) {
    cplxf v;
    asm volatile("ld.relaxed.cluster.f32 %0, [%1];" : "=f"(v.x) : "l"(a) : "memory");
    asm volatile("ld.relaxed.cluster.f32 %0, [%1];" : "=f"(v.y) : "l"(a + 4) : "memory");
    return v;
}

template <typename T>
__device__ __forceinline__ T ld_l2(const T *p) {
    return __ldcg(p);
}
template <>
__device__ __forceinline__ cplx ld_l2<cplx>(const cplx *p) {
    const double2 v = __ldcg((const double2 *)p);
    return {v.x, v.y};
}
template <>
__device__ __forceinline__ cplxf ld_l2<cplxf>(const cplxf *p) {
    const float2 v = __ldcg((const float2 *)p);
    return {v.x, v.y};
}

// shared-memory carve-up, identical on host and device
struct ClLayout {
    int S;      // ring slots (values)
    int cap_r;  // rows of the largest per-CTA chunk of a level
    int cap_e;  // entries of the largest per-CTA chunk of a level
    int ring2;  // second ring for the fused Eisenstat output (0/1)
    int ngath;  // gathered per-row inputs (1 or 2)
    // byte offsets
    int o_ring, o_ring2, o_span, span_bytes, o_codes, o_vals, o_prp, o_perm, o_lvec, o_gath, gath_bytes, o_tab, o_prog,
        total;
};

__host__ __device__ inline int al16(int x) { return (x + 15) & ~15; }

__host__ __device__ inline ClLayout cl_layout(int S, int cap_r, int cap_e, int elem, int ring2, int ngath, int nlev) {
    ClLayout L;
    L.S = S;
    L.cap_r = cap_r;
    L.cap_e = cap_e;
    L.ring2 = ring2;
    L.ngath = ngath;
    int o = 0;
    L.o_ring = o;
    o += al16(S * elem);
    L.o_ring2 = o;
    if (ring2) o += al16(S * elem);
    L.o_span = o;
    int so = 0;
    L.o_codes = so;
    so += al16((cap_e + 2 * CL_PAD) * 4);
    L.o_vals = so;
    so += al16((cap_e + 2 * CL_PAD) * elem);
    L.o_prp = so;
    so += al16((cap_r + 1) * 4);
    L.o_perm = so;
    so += al16(cap_r * 4);
    L.o_lvec = so;
    so += al16(cap_r * elem);
    L.span_bytes = so;
    o += CL_SPAN_BUFS * so;
    L.o_gath = o;
    L.gath_bytes = al16(cap_r * elem * ngath);
    o += CL_GATH_BUFS * L.gath_bytes;
    L.o_tab = o;  // per level: this CTA's chunk (see cluster_plan for the packing)
    o += al16(nlev * 16);
    L.o_prog = o;  // neighbour-synchronised sweep: progress word
    o += 16;
    L.total = o;
    return L;
}

// P2P: neighbour-synchronised. No cluster barrier per level: the store warp
// publishes the CTA's progress (a release on a shared-memory word) and, before
// the next level, waits (bounded) until every CTA this chunk reads from has
// published the levels it needs and no CTA is more than CL_LEAD levels behind.
template <typename T, int G, int MODE, bool P2P>
__global__ void __launch_bounds__(544) k_sweep_cluster(int nlev, int ncomp, const int *__restrict__ lptr,
                                                        const int *__restrict__ perm, const int *__restrict__ prp,
                                                        const int *__restrict__ code, const T *__restrict__ val,
                                                        const T *__restrict__ lvec, const T *rhs, const T *aux, T *out,
                                                        T *out2, const KState *st, const int4 *__restrict__ tab,
                                                        int *err, ClLayout Lay) {
    if (st && !st->active) return;  // uniform across the cluster
    extern __shared__ __align__(16) unsigned char cl_smem[];
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(cl_smem);
    T *ring = (T *)(cl_smem + Lay.o_ring);
    T *ring2 = (T *)(cl_smem + Lay.o_ring2);
    const int C = (int)cluster_size();
    const int rank = (int)cluster_rank();
    const int tid = threadIdx.x;
    const bool is_store = tid >= ncomp;
    const int nthreads = blockDim.x;
    const int NG = ncomp / G;
    const int g = tid / G, gl = tid % G;
    constexpr bool fwd = (MODE == SW_FWD_DIV || MODE == SW_FWD_EIS);
    constexpr bool eis = (MODE == SW_FWD_EIS);
    constexpr int VB = (int)sizeof(T);

    // this CTA's chunk of every level, staged once: no global index loads inside the level loop
    int4 *s_tab = (int4 *)(cl_smem + Lay.o_tab);
    for (int q = tid; q < nlev; q += nthreads) s_tab[q] = __ldg(tab + (size_t)q * C + rank);
    __syncthreads();
    // table entry: x = first row, y = rows | producer mask << 16, z = first entry,
    // w = entries | (level - required progress) << 16 (signed)
    auto chunk_of = [&](int l, int &rs, int &re) {
        const int4 c4 = s_tab[l];
        rs = c4.x;
        re = c4.x + (c4.y & 0xFFFF);
    };
    auto span_base = [&](int l) { return Lay.o_span + (l % CL_SPAN_BUFS) * Lay.span_bytes; };
    auto gath_base = [&](int l) { return Lay.o_gath + (l % CL_GATH_BUFS) * Lay.gath_bytes; };
    // stage the matrix span of level l: entry codes and values (16-byte copies of the
    // aligned superset of [e0, e1); the arrays carry CL_PAD entries of padding), row
    // pointers, row ids, per-row vector
    constexpr int CPE = 16 / 4;              // codes per 16-byte copy
    constexpr int VPE = VB >= 16 ? 1 : 16 / VB;  // values per 16-byte copy
    auto stage_span = [&](int l) {
        if (l >= nlev || is_store) return;
        int rs, re;
        chunk_of(l, rs, re);
        const int cnt = re - rs;
        if (cnt <= 0) return;
        const int e0 = s_tab[l].z, e1 = s_tab[l].z + (s_tab[l].w & 0xFFFF);
        const int sb = span_base(l);
        const int c0 = e0 & ~(CPE - 1), v0 = e0 & ~(VPE - 1);
        for (int i = tid; i * CPE < e1 - c0; i += ncomp)
            cp_async<16>(sbase + sb + Lay.o_codes + 16 * i, code + c0 + CPE * i);
        for (int i = tid; i * VPE < e1 - v0; i += ncomp)
            cp_async<16>(sbase + sb + Lay.o_vals + 16 * i, val + v0 + VPE * i);
        for (int i = tid; i <= cnt; i += ncomp) cp_async<4>(sbase + sb + Lay.o_prp + 4 * i, prp + rs + i);
        for (int i = tid; i < cnt; i += ncomp) {
            cp_async<4>(sbase + sb + Lay.o_perm + 4 * i, perm + rs + i);
            if (lvec) cp_async<VB>(sbase + sb + Lay.o_lvec + VB * i, lvec + rs + i);
        }
    };
    // gather level l's per-row inputs (rhs and/or aux by row id); its span must be staged
    auto stage_gath = [&](int l) {
        if (l >= nlev || is_store) return;
        int rs, re;
        chunk_of(l, rs, re);
        const int cnt = re - rs;
        const int *sperm = (const int *)(cl_smem + span_base(l) + Lay.o_perm);
        const int gb = gath_base(l);
        for (int i = tid; i < cnt; i += ncomp) {
            const int r = sperm[i];
            if (MODE == SW_BWD_IC) {
                cp_async<VB>(sbase + gb + VB * i, aux + r);
            } else {
                cp_async<VB>(sbase + gb + VB * i, rhs + r);
                if (eis) cp_async<VB>(sbase + gb + VB * (Lay.cap_r + i), aux + r);
            }
        }
    };

    if (P2P) {
        // every CTA's progress word is zero before any CTA reads another's
        if (tid == 0) *(volatile unsigned *)(cl_smem + Lay.o_prog) = 0u;
        cluster_arrive_release();
        cluster_wait_acquire();
    }
    // prologue: spans of levels 0..3, then gathers of levels 0..1
    for (int q = 0; q < CL_SPAN_BUFS - 1; ++q) stage_span(q);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    stage_gath(0);
    stage_gath(1);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();

    int produced = 0;  // values this CTA has written to its ring so far
    for (int l = 0; l < nlev; ++l) {
        // A: every copy group but the two newest (the gathers of l+1 and the span of
        // l+3, issued one level ago) has landed: the span of l+2 and the gathers of l
        // are complete and visible CTA-wide
        cp_async_wait_prev2();
        __syncthreads();
        int rs, re;
        chunk_of(l, rs, re);
        const int cnt = re - rs;
        const unsigned char *sp = cl_smem + span_base(l);
        const int *sprp = (const int *)(sp + Lay.o_prp);
        const int e0l = cnt > 0 ? sprp[0] : 0;
        // entry k of the span (0-based from e0) sits at k + (e0 - aligned start) in the staged copies
        const int *scode = (const int *)(sp + Lay.o_codes) + (e0l & (CPE - 1));
        const T *sval = (const T *)(sp + Lay.o_vals) + (e0l & (VPE - 1));
        const int *sperm = (const int *)(sp + Lay.o_perm);
        const T *slvec = (const T *)(sp + Lay.o_lvec);
        const T *sg = (const T *)(cl_smem + gath_base(l));
        if (!is_store) {
            // B: solve the rows of this level
            const unsigned gm = group_mask(G);
            const int base_e = cnt > 0 ? sprp[0] : 0;
            for (int q = g; q < cnt; q += NG) {
                const int a = sprp[q] - base_e, e = sprp[q + 1] - base_e;
                const int ob = fwd ? a : a + 1;
                const int oe = fwd ? (e > a ? e - 1 : a) : e;
                // IC pair: the sum is taken negated, and the forward right-hand side starts
                // lane 0's sum, so the row's result is one operation after the reduction
                // (the same arithmetic as the sync-free sweep)
                constexpr bool neg = (MODE == SW_FWD_DIV || MODE == SW_BWD_IC);
                T acc = (MODE == SW_FWD_DIV && gl == 0 && q < cnt) ? sg[q] : Sc<T>::zero();
                // four entries per step: all addresses first, then all loads, then the
                // multiply-adds in entry order (the same order as the sync-free sweep)
                for (int k0 = ob + gl; k0 < oe; k0 += 4 * G) {
                    unsigned long long ad[4];
                    T vv[4], xx[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int k = k0 + u * G;
                        if (k < oe) {
                            const int cd = scode[k];
                            vv[u] = sval[k];
                            const int sl = -1 - cd;
                            ad[u] = cd >= 0 ? (unsigned long long)(out + cd)
                                            : mapa_generic(ring + (sl & ((1 << CL_SLOT_BITS) - 1)),
                                                           (unsigned)(sl >> CL_SLOT_BITS));
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (k0 + u * G < oe) xx[u] = ld_rc<T>(ad[u]);
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (k0 + u * G < oe) acc = madd(acc, neg ? -vv[u] : vv[u], xx[u]);
                }
#pragma unroll
                for (int m = G / 2; m >= 1; m >>= 1) acc = acc + gshfl_xor(acc, m, gm);
                if (gl == 0) {
                    T res;
                    if (MODE == SW_BWD_IC) {
                        res = madd(sg[q], slvec[q], acc);  // aux + D * (-sum)
                    } else if (MODE == SW_FWD_DIV) {
                        res = lvec ? acc * slvec[q] : acc / ((e > a) ? sval[e - 1] : Sc<T>::zero());
                    } else {
                        T num = sg[q] - acc;
                        T u = Sc<T>::zero();
                        if (eis) {
                            u = sg[Lay.cap_r + q];
                            num = (sg[q] - u) - acc;
                        }
                        if (lvec) res = num * slvec[q];
                        else res = num / ((e > a) ? sval[fwd ? e - 1 : a] : Sc<T>::zero());
                        if (eis) ring2[(produced + q) % Lay.S] = res + u;
                    }
                    ring[(produced + q) % Lay.S] = res;
                }
            }
            // results are in the ring: let the store warp copy them out
            bar_arrive(1, nthreads);
            if (P2P) {
                // publish: the compute warps have only shared-memory stores pending,
                // so this release is short
                bar_sync(2, ncomp);
                if (tid == 0) st_release_progress(sbase + Lay.o_prog, (unsigned)(l + 1));
            } else {
                cluster_arrive_release();
            }
            // C: stage the gathers of level l+2 (its span landed) and the span of level l+4
            // while the barrier completes: two groups, the span one newest
            stage_gath(l + 2);
            cp_async_commit();
            stage_span(l + CL_SPAN_BUFS - 1);
            cp_async_commit();
            if (!P2P) cluster_wait_acquire();
        } else {
            bar_sync(1, nthreads);
            if (!P2P) {
                // release at every K-th level publishes the stores of the earlier levels
                if (l % CL_STORE_K == 0) cluster_arrive_release();
                else cluster_arrive_relaxed();
            }
            for (int i = tid - ncomp; i < cnt; i += nthreads - ncomp) {
                const int r = sperm[i];
                out[r] = ring[(produced + i) % Lay.S];
                if (eis) out2[r] = ring2[(produced + i) % Lay.S];
            }
            if (!P2P) {
                cluster_wait_acquire();
            } else if (l + 1 < nlev) {
                // before level l+1: the CTAs it reads from have published what it needs,
                // and no CTA is more than CL_LEAD levels behind (its ring entries stay
                // valid); lane q watches CTA q, bounded in time
                const int q = tid - ncomp;
                if (q < C && q != rank) {
                    const int4 nx = s_tab[l + 1];
                    const int mask = (nx.y >> 16) & 0xFFFF;
                    const int delta = nx.w >> 16;  // level - required progress (signed)
                    int req = ((mask >> q) & 1) ? (l + 1) - delta : 0;
                    req = max(req, (l + 1) - CL_LEAD);
                    if (req > 0) {
                        const unsigned ra = map_shared(sbase + Lay.o_prog, (unsigned)q);
                        if ((int)ld_acquire_progress(ra) < req) {
                            const unsigned long long t0 = gtimer();
                            int polls = 0;
                            while ((int)ld_acquire_progress(ra) < req) {
                                if ((++polls & 63) == 0) {
                                    if (*(volatile int *)err) break;
                                    if (gtimer() - t0 > spin_limit_ns(err)) {
                                        atomicExch(err, ERR_TIMEOUT);
                                        break;
                                    }
                                }
                            }
                        }
                    }
                }
                __syncwarp();
            }
        }
        produced += cnt;
    }
    if (P2P) {
        // no CTA leaves while another may still read its shared memory
        cluster_arrive_release();
        cluster_wait_acquire();
    }
}

// ---------------------------------------------------------------- plan
// per position p of the level order: owner CTA and production index
__global__ void k_cl_positions(int n, const int *perm, const int *level, const int *lptr, const int *end_ord,
                               int C, unsigned char *owner, int *ord) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int l = level[perm[p]];
    const int L0 = lptr[l], L1 = lptr[l + 1];
    const int chunk = (L1 - L0 + C - 1) / C;
    const int off = p - L0;
    const int c = off / chunk;
    owner[p] = (unsigned char)c;
    ord[p] = (l > 0 ? end_ord[(l - 1) * C + c] : 0) + (off - c * chunk);
}

// per entry: ring (owner, slot) when still resident, memory index when published, else infeasible
__global__ void k_cl_codes(int n, const int *perm, const int *level, const int *prp, const int *pci, const int *ipos,
                           const unsigned char *owner, const int *ord, const int *end_ord, int C, int S, int K,
                           int *code, int *infeasible) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int lt = level[perm[t]];
    for (int k = prp[t]; k < prp[t + 1]; ++k) {
        const int j = pci[k];
        const int lj = level[j];
        if (lj >= lt) {  // the row itself (diagonal): never read as a dependency
            code[k] = j;
            continue;
        }
        const int p = ipos[j];
        const int c = owner[p];
        const int o = ord[p];
        const int written = end_ord[lt * C + c];  // values of c in its ring by the end of level lt
        // the first release covering the stores of level lj: the arrive of the
        // first level after lj that is a multiple of K; seen by levels after it
        const int rel = (lj / K + 1) * K;
        if (written - o <= S) code[k] = -1 - ((c << CL_SLOT_BITS) | (o % S));
        else if (rel <= lt - 1) code[k] = j;
        else {
            code[k] = j;
            atomicExch(infeasible, 1);
        }
    }
}

// neighbour-synchronised plan: every dependency on another CTA must sit in that
// CTA's ring even when the producer is CL_LEAD levels ahead (else infeasible);
// own values older than the ring are read from memory (stored by this CTA's
// store warp before any later level starts). Per (level, CTA): the producers
// read (mask) and the progress they must have published (the largest level read + 1).
__global__ void k_cl_codes_p2p(int n, const int *perm, const int *level, const int *prp, const int *pci,
                               const int *ipos, const unsigned char *owner, const int *ord, const int *end_ord, int C,
                               int S, int nlev, int *code, int *needmask, int *needreq, int *infeasible) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int lt = level[perm[t]];
    const int cons = owner[t];
    for (int k = prp[t]; k < prp[t + 1]; ++k) {
        const int j = pci[k];
        const int lj = level[j];
        if (lj >= lt) {
            code[k] = j;
            continue;
        }
        const int p = ipos[j];
        const int c = owner[p];
        const int o = ord[p];
        if (c == cons) {
            const int written = end_ord[lt * C + c];
            code[k] = (written - o <= S) ? -1 - ((c << CL_SLOT_BITS) | (o % S)) : j;
        } else {
            const int lk = min(lt + CL_LEAD, nlev - 1);
            const int written = end_ord[lk * C + c];
            if (written - o <= S) {
                code[k] = -1 - ((c << CL_SLOT_BITS) | (o % S));
                atomicOr(needmask + lt * C + cons, 1 << c);
                atomicMax(needreq + lt * C + cons, lj + 1);
            } else {
                code[k] = j;
                atomicExch(infeasible, 1);
            }
        }
    }
}

static int g_cluster_size = -1;

template <typename T>
static int probe_cluster(int smem) {
    auto kern = k_sweep_cluster<T, 4, SW_FWD_DIV, false>;
    for (int C : {16, 8}) {
        if (C > 8) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
                (void)cudaGetLastError();
                continue;
            }
        }
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) {
            (void)cudaGetLastError();
            return 0;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(C);
        cfg.blockDim = dim3(544);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = C;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess && nclusters > 0) return C;
        (void)cudaGetLastError();
    }
    return 0;
}

constexpr int CL_SMEM_MAX = 220 * 1024;

int cluster_size_available() {
    if (g_cluster_size < 0) g_cluster_size = probe_cluster<double>(CL_SMEM_MAX);
    return g_cluster_size;
}

void cluster_plan(Tri &T, size_t elem_bytes, int ring_bytes, cudaStream_t s, DBuf &tmp, bool p2p) {
    (void)tmp;
    T.cl_ready = false;
    if (T.n == 0) return;
    const int C = cluster_size_available();
    if (C <= 0) return;
    const int nlev = T.nlev;
    // end_ord[l][c]: values CTA c has produced by the end of level l; the largest chunk
    std::vector<int> end_ord((size_t)nlev * C);
    std::vector<int> run(C, 0);
    int cap_r = 1;
    for (int l = 0; l < nlev; ++l) {
        const int L0 = T.lptr[l], L1 = T.lptr[l + 1];
        const int chunk = (L1 - L0 + C - 1) / C;
        cap_r = std::max(cap_r, chunk);
        for (int c = 0; c < C; ++c) {
            const int rs = std::min(L0 + c * chunk, L1), re = std::min(rs + chunk, L1);
            run[c] += re - rs;
            end_ord[(size_t)l * C + c] = run[c];
        }
    }
    // largest entry span of a chunk (needs the row pointers)
    std::vector<int> prp(T.n + 1);
    SSG_CUDA(cudaMemcpyAsync(prp.data(), T.prp.p, sizeof(int) * (size_t)(T.n + 1), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaStreamSynchronize(s));
    // table entry per (level, CTA): x = first row, y = rows | producer mask << 16,
    // z = first entry, w = entries | (level - required progress) << 16; the mask and
    // the requirement are filled for the neighbour-synchronised sweep
    int cap_e = 1;
    std::vector<int4> tab((size_t)nlev * C);
    for (int l = 0; l < nlev; ++l) {
        const int L0 = T.lptr[l], L1 = T.lptr[l + 1];
        const int chunk = (L1 - L0 + C - 1) / C;
        for (int c = 0; c < C; ++c) {
            const int rs = std::min(L0 + c * chunk, L1), re = std::min(rs + chunk, L1);
            cap_e = std::max(cap_e, prp[re] - prp[rs]);
            tab[(size_t)l * C + c] = make_int4(rs, re - rs, prp[rs], prp[re] - prp[rs]);
        }
    }
    if (cap_r > 0xFFFF || cap_e > 0xFFFF) return;  // the packed table holds 16-bit counts
    const int elem = (int)elem_bytes;
    // sized for the fused Eisenstat sweep (second ring, two gathered inputs), the largest
    // mode; the neighbour-synchronised plan serves the IC sweeps only
    const ClLayout lay = p2p ? cl_layout(ring_bytes / elem, cap_r, cap_e, elem, 0, 1, nlev)
                             : cl_layout(ring_bytes / elem, cap_r, cap_e, elem, 1, 2, nlev);
    if (T.nnz_pad < CL_PAD) return;  // the value arrays must carry padding for the aligned copies
    if (lay.total > CL_SMEM_MAX || lay.S >= (1 << CL_SLOT_BITS)) return;  // sync-free sweep instead
    const int S = lay.S;
    DBuf eo, owner, ord, inf;
    eo.alloc(sizeof(int) * end_ord.size());
    SSG_CUDA(cudaMemcpyAsync(eo.p, end_ord.data(), sizeof(int) * end_ord.size(), cudaMemcpyHostToDevice, s));
    owner.alloc((size_t)T.n);
    ord.alloc(sizeof(int) * (size_t)T.n);
    inf.alloc(sizeof(int));
    SSG_CUDA(cudaMemsetAsync(inf.p, 0, sizeof(int), s));
    k_cl_positions<<<div_up(T.n, 256), 256, 0, s>>>(T.n, T.perm.as<int>(), T.level.as<int>(), T.lptr_d.as<int>(),
                                                   eo.as<int>(), C, owner.as<unsigned char>(), ord.as<int>());
    SSG_LAUNCHED();
    T.cl_code.ensure(sizeof(int) * (size_t)(T.nnz + T.nnz_pad));
    SSG_CUDA(cudaMemsetAsync(T.cl_code.p, 0, sizeof(int) * (size_t)(T.nnz + T.nnz_pad), s));
    if (p2p) {
        DBuf nm, nr;
        nm.alloc(sizeof(int) * tab.size());
        nr.alloc(sizeof(int) * tab.size());
        SSG_CUDA(cudaMemsetAsync(nm.p, 0, sizeof(int) * tab.size(), s));
        SSG_CUDA(cudaMemsetAsync(nr.p, 0, sizeof(int) * tab.size(), s));
        k_cl_codes_p2p<<<div_up(T.n, 256), 256, 0, s>>>(
            T.n, T.perm.as<int>(), T.level.as<int>(), T.prp.as<int>(), T.pci.as<int>(), T.ipos.as<int>(),
            owner.as<unsigned char>(), ord.as<int>(), eo.as<int>(), C, S, nlev, T.cl_code.as<int>(), nm.as<int>(),
            nr.as<int>(), inf.as<int>());
        SSG_LAUNCHED();
        std::vector<int> hm(tab.size()), hr(tab.size());
        SSG_CUDA(cudaMemcpyAsync(hm.data(), nm.p, sizeof(int) * tab.size(), cudaMemcpyDeviceToHost, s));
        SSG_CUDA(cudaMemcpyAsync(hr.data(), nr.p, sizeof(int) * tab.size(), cudaMemcpyDeviceToHost, s));
        SSG_CUDA(cudaStreamSynchronize(s));
        for (int l = 0; l < nlev; ++l)
            for (int c = 0; c < C; ++c) {
                const size_t q = (size_t)l * C + c;
                if (!hm[q]) continue;
                const int delta = std::min(l - hr[q], 0x7FFF);  // >= 0: a dependency is an earlier level
                tab[q].y |= hm[q] << 16;
                tab[q].w |= delta << 16;
            }
    } else {
        k_cl_codes<<<div_up(T.n, 256), 256, 0, s>>>(T.n, T.perm.as<int>(), T.level.as<int>(), T.prp.as<int>(),
                                                    T.pci.as<int>(), T.ipos.as<int>(), owner.as<unsigned char>(),
                                                    ord.as<int>(), eo.as<int>(), C, S, CL_STORE_K,
                                                    T.cl_code.as<int>(), inf.as<int>());
        SSG_LAUNCHED();
    }
    T.cl_tab.ensure(sizeof(int4) * tab.size());
    SSG_CUDA(cudaMemcpyAsync(T.cl_tab.p, tab.data(), sizeof(int4) * tab.size(), cudaMemcpyHostToDevice, s));
    int infeasible = 0;
    SSG_CUDA(cudaMemcpyAsync(&infeasible, inf.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    SSG_CUDA(cudaStreamSynchronize(s));
    if (infeasible) return;
    T.cl_p2p = p2p;
    T.cl_C = C;
    T.cl_S = S;
    T.cl_elem = elem;
    T.cl_ring_bytes = ring_bytes;
    T.cl_cap_r = cap_r;
    T.cl_cap_e = cap_e;
    T.cl_ready = true;
}

template <typename T, int G, bool P2P>
static void launch_cluster(const Tri &tri, const T *val, int mode, const T *rhs, const T *aux, const T *lvec, T *out,
                           T *out2, const KState *st, int *err, cudaStream_t s) {
    const int elem = (int)sizeof(T);
    const ClLayout lay = cl_layout(tri.cl_S, tri.cl_cap_r, tri.cl_cap_e, elem, mode == SW_FWD_EIS ? 1 : 0,
                                   mode == SW_FWD_EIS ? 2 : 1, tri.nlev);
    // compute threads: enough groups for the widest chunk, 64..512, plus one store warp
    int ncomp = std::min(512, std::max(64, ((tri.cl_cap_r * G + 31) / 32) * 32));
    ncomp = (ncomp / G) * G;
    const int nthreads = ncomp + 32;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(tri.cl_C);
    cfg.blockDim = dim3(nthreads);
    cfg.dynamicSmemBytes = lay.total;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = tri.cl_C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const int *lp = tri.lptr_d.as<int>(), *pm = tri.perm.as<int>(), *pr = tri.prp.as<int>(),
              *cd = tri.cl_code.as<int>();
#define SSG_CL(M)                                                                                                \
    do {                                                                                                         \
        auto kern = k_sweep_cluster<T, G, M, P2P>;                                                               \
        static bool prepared = false;                                                                            \
        if (!prepared) {                                                                                         \
            if (tri.cl_C > 8)                                                                                    \
                SSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));         \
            SSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, CL_SMEM_MAX));      \
            prepared = true;                                                                                     \
        }                                                                                                        \
        SSG_CUDA(cudaLaunchKernelEx(&cfg, kern, tri.nlev, ncomp, lp, pm, pr, cd, val, lvec, rhs, aux, out, out2, \
                                    st, tri.cl_tab.as<int4>(), err, lay));                                       \
    } while (0)
    if (P2P) {
        // the neighbour-synchronised plan serves the IC sweeps
        switch (mode) {
            case SW_FWD_DIV: SSG_CL(SW_FWD_DIV); break;
            case SW_BWD_IC: SSG_CL(SW_BWD_IC); break;
            default: throw Error{SSG_ERR_STATE, "neighbour-synchronised plan used for a non-IC sweep"};
        }
    } else {
        switch (mode) {
            case SW_FWD_DIV: SSG_CL(SW_FWD_DIV); break;
            case SW_BWD_IC: SSG_CL(SW_BWD_IC); break;
            case SW_BWD_DIV: SSG_CL(SW_BWD_DIV); break;
            default: SSG_CL(SW_FWD_EIS); break;
        }
    }
#undef SSG_CL
}

template <typename T>
void sweep_cluster(const Tri &tri, const T *val, int mode, const T *rhs, const T *aux, const T *lvec, T *out, T *out2,
                   const KState *st, int group, int *err, cudaStream_t s) {
    if (tri.n == 0) return;
    const int G = group ? group : sweep_group(tri);
    if (tri.cl_p2p) {
        // neighbour-synchronised kernels exist for 4 and 8 lanes a row
        if (G == 8)
            launch_cluster<T, 8, true>(tri, val, mode, rhs, aux, lvec, out, out2, st, err, s);
        else if (G == 4)
            launch_cluster<T, 4, true>(tri, val, mode, rhs, aux, lvec, out, out2, st, err, s);
        else
            throw Error{SSG_ERR_ARG, "the neighbour-synchronised sweep runs with 4 or 8 lanes a row"};
    } else if (G == 8)
        launch_cluster<T, 8, false>(tri, val, mode, rhs, aux, lvec, out, out2, st, err, s);
    else if (G == 16)
        launch_cluster<T, 16, false>(tri, val, mode, rhs, aux, lvec, out, out2, st, err, s);
    else if (G == 32)
        launch_cluster<T, 32, false>(tri, val, mode, rhs, aux, lvec, out, out2, st, err, s);
    else
        launch_cluster<T, 4, false>(tri, val, mode, rhs, aux, lvec, out, out2, st, err, s);
    SSG_LAUNCHED();
}

#define SSG_INST(T)                                                                                        \
    template void sweep_cluster<T>(const Tri &, const T *, int, const T *, const T *, const T *, T *, T *, \
                                   const KState *, int, int *, cudaStream_t);
SSG_INST(double)
SSG_INST(cplx)
SSG_INST(float)
SSG_INST(cplxf)
#undef SSG_INST

}  // namespace ssg
