// ss_cluster.cu -- level-synchronous triangular sweeps inside one thread-block
// cluster, with recent results exchanged through distributed shared memory.
//
// The sync-free sweep (ss_trsv.cu) pays several L2 round trips per dependency
// level (publish, poll, gather). Here one cluster of C CTAs (C = 16 where the
// GPU allows non-portable cluster sizes, else 8) runs the whole sweep:
//   for each level l:  every CTA solves its contiguous share of the level's
//                      rows, writes each result to the output vector in HBM
//                      and to its own shared-memory ring; then all CTAs meet
//                      at a cluster barrier (release / acquire).
// A dependency produced within the last few levels is read from the
// producing CTA's ring with ld.shared::cluster; older ones from L2. Which of
// the two applies, and the (CTA, slot) of a ring entry, are integer facts of
// the pattern computed once (ClusterPlan): entry k of the level-ordered
// triangle carries code[k] = j (read out[j] from memory) or
// -1 - (owner << 20 | slot). A slot is only used when no later value of the
// owner can have overwritten it before the consumer's level ends.
// There is no spin-wait at all: the only waits are cluster barriers, which
// every CTA reaches the same number of times.
#include <algorithm>

#include "ss_internal.cuh"
#include "ss_krylov.cuh"

namespace ssg {

constexpr int CL_THREADS = 512;
constexpr int CL_SLOT_BITS = 20;

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
__device__ __forceinline__ void cluster_wait_acquire() {
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
__device__ __forceinline__ unsigned map_shared(unsigned local_addr, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local_addr), "r"(rank));
    return r;
}
template <typename T>
__device__ __forceinline__ T ld_dsmem(unsigned addr);
template <>
__device__ __forceinline__ double ld_dsmem<double>(unsigned addr) {
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
    return v;
}
template <>
__device__ __forceinline__ float ld_dsmem<float>(unsigned addr) {
    float v;
    asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr) : "memory");
    return v;
}
template <>
__device__ __forceinline__ cplx ld_dsmem<cplx>(unsigned addr) {
    cplx v;
    asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(addr) : "memory");
    return v;
}
template <>
__device__ __forceinline__ cplxf ld_dsmem<cplxf>(unsigned addr) {
    cplxf v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr) : "memory");
    return v;
}
template <typename T>
__device__ __forceinline__ T ld_ro(const T *p) {
    return __ldg(p);
}
template <>
__device__ __forceinline__ cplx ld_ro<cplx>(const cplx *p) {
    const double2 v = __ldg((const double2 *)p);
    return {v.x, v.y};
}
template <>
__device__ __forceinline__ cplxf ld_ro<cplxf>(const cplxf *p) {
    const float2 v = __ldg((const float2 *)p);
    return {v.x, v.y};
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

template <typename T, int G, int MODE>
__global__ void __launch_bounds__(CL_THREADS) k_sweep_cluster(int nlev, const int *__restrict__ lptr,
                                                              const int *__restrict__ perm,
                                                              const int *__restrict__ prp,
                                                              const int *__restrict__ code,
                                                              const T *__restrict__ val, const T *rhs, const T *aux,
                                                              const T *D, T *out, T *out2, const T *dinv,
                                                              const KState *st, int ring_cap) {
    if (st && !st->active) return;  // uniform across the cluster
    extern __shared__ __align__(16) unsigned char cl_smem[];
    T *ring = (T *)cl_smem;
    const unsigned ring_base = (unsigned)__cvta_generic_to_shared(ring);
    const int C = (int)cluster_size();
    const int rank = (int)cluster_rank();
    constexpr int NG = CL_THREADS / G;
    const int g = threadIdx.x / G, gl = threadIdx.x % G;
    const unsigned gm = group_mask(G);
    const bool fwd = (MODE == SW_FWD_DIV || MODE == SW_FWD_EIS);
    int produced = 0;  // values this CTA has written to its ring so far
    for (int l = 0; l < nlev; ++l) {
        const int L0 = __ldg(lptr + l), L1 = __ldg(lptr + l + 1);
        const int chunk = (L1 - L0 + C - 1) / C;
        const int rs = min(L0 + rank * chunk, L1), re = min(rs + chunk, L1);
        for (int t = rs + g; t < re; t += NG) {
            const int r = __ldg(perm + t);
            const int a = __ldg(prp + t), e = __ldg(prp + t + 1);
            const int ob = fwd ? a : a + 1;
            const int oe = fwd ? (e > a ? e - 1 : a) : e;
            T acc = Sc<T>::zero();
#pragma unroll 2
            for (int k = ob + gl; k < oe; k += G) {
                const int cd = __ldg(code + k);
                const T v = ld_ro(val + k);
                T x;
                if (cd >= 0) {
                    x = ld_l2(out + cd);
                } else {
                    const int s = -1 - cd;
                    x = ld_dsmem<T>(map_shared(ring_base + (unsigned)((s & ((1 << CL_SLOT_BITS) - 1)) * sizeof(T)),
                                               (unsigned)(s >> CL_SLOT_BITS)));
                }
                acc = acc + v * x;
            }
#pragma unroll
            for (int m = G / 2; m >= 1; m >>= 1) acc = acc + gshfl_xor(acc, m, gm);
            if (gl == 0) {
                T res;
                if (MODE == SW_BWD_IC) {
                    res = D[r] * (Sc<T>::zero() - acc) + aux[r];
                } else {
                    T num = rhs[r] - acc;
                    T u = Sc<T>::zero();
                    if (MODE == SW_FWD_EIS) {
                        u = aux[r];
                        num = (rhs[r] - u) - acc;
                    }
                    if (dinv) res = num * dinv[r];
                    else res = num / ((e > a) ? val[fwd ? e - 1 : a] : Sc<T>::zero());
                    if (MODE == SW_FWD_EIS) out2[r] = res + u;
                }
                out[r] = res;
                ring[(produced + (t - rs)) % ring_cap] = res;
            }
        }
        produced += re - rs;
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

// per entry: ring (owner, slot) when still resident during the consumer's level, else the row id
__global__ void k_cl_codes(int n, const int *perm, const int *level, const int *prp, const int *pci, const int *ipos,
                           const unsigned char *owner, const int *ord, const int *end_ord, int C, int S,
                           int *code) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int lt = level[perm[t]];
    for (int k = prp[t]; k < prp[t + 1]; ++k) {
        const int j = pci[k];
        const int p = ipos[j];
        const int c = owner[p];
        const int o = ord[p];
        const int written = end_ord[lt * C + c];  // values of c written by the end of level lt
        code[k] = (level[j] < lt && written - o <= S) ? -1 - ((c << CL_SLOT_BITS) | (o % S)) : j;
    }
}

static int g_cluster_size = -1;

// largest cluster the device schedules for this kernel shape (16 or 8), 0 if none
template <typename T>
static int probe_cluster(int smem) {
    auto kern = k_sweep_cluster<T, 16, SW_FWD_DIV>;
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
        cfg.blockDim = dim3(CL_THREADS);
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

void cluster_plan(Tri &T, size_t elem_bytes, int ring_bytes, cudaStream_t s, DBuf &tmp) {
    T.cl_ready = false;
    if (T.n == 0) return;
    if (g_cluster_size < 0) g_cluster_size = probe_cluster<double>(ring_bytes);
    const int C = g_cluster_size;
    if (C <= 0) return;
    const int nlev = T.nlev;
    const int S = ring_bytes / (int)elem_bytes;
    // end_ord[l][c]: values CTA c has produced by the end of level l
    std::vector<int> end_ord((size_t)nlev * C);
    std::vector<int> run(C, 0);
    for (int l = 0; l < nlev; ++l) {
        const int L0 = T.lptr[l], L1 = T.lptr[l + 1];
        const int chunk = (L1 - L0 + C - 1) / C;
        for (int c = 0; c < C; ++c) {
            const int rs = std::min(L0 + c * chunk, L1), re = std::min(rs + chunk, L1);
            run[c] += re - rs;
            end_ord[(size_t)l * C + c] = run[c];
        }
    }
    DBuf eo, owner, ord;
    eo.alloc(sizeof(int) * end_ord.size());
    SSG_CUDA(cudaMemcpyAsync(eo.p, end_ord.data(), sizeof(int) * end_ord.size(), cudaMemcpyHostToDevice, s));
    owner.alloc((size_t)T.n);
    ord.alloc(sizeof(int) * (size_t)T.n);
    k_cl_positions<<<div_up(T.n, 256), 256, 0, s>>>(T.n, T.perm.as<int>(), T.level.as<int>(), T.lptr_d.as<int>(),
                                                   eo.as<int>(), C, owner.as<unsigned char>(), ord.as<int>());
    SSG_LAUNCHED();
    T.cl_code.ensure(sizeof(int) * (size_t)(T.nnz + 1));
    k_cl_codes<<<div_up(T.n, 256), 256, 0, s>>>(T.n, T.perm.as<int>(), T.level.as<int>(), T.prp.as<int>(),
                                                T.pci.as<int>(), T.ipos.as<int>(), owner.as<unsigned char>(),
                                                ord.as<int>(), eo.as<int>(), C, S, T.cl_code.as<int>());
    SSG_LAUNCHED();
    SSG_CUDA(cudaStreamSynchronize(s));
    T.cl_C = C;
    T.cl_S = S;
    T.cl_elem = (int)elem_bytes;
    T.cl_ring_bytes = ring_bytes;
    T.cl_ready = true;
    (void)tmp;
}

template <typename T, int G>
static void launch_cluster(const Tri &tri, const T *val, int mode, const T *rhs, const T *aux, const T *D, T *out,
                           T *out2, const T *dinv, const KState *st, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(tri.cl_C);
    cfg.blockDim = dim3(CL_THREADS);
    cfg.dynamicSmemBytes = tri.cl_ring_bytes;
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
    const int ring_cap = tri.cl_S;
#define SSG_CL(M)                                                                                       \
    do {                                                                                                \
        auto kern = k_sweep_cluster<T, G, M>;                                                           \
        static int prepared_bytes = -1;                                                                 \
        if (prepared_bytes != tri.cl_ring_bytes) {                                                      \
            if (tri.cl_C > 8) SSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)); \
            SSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, tri.cl_ring_bytes)); \
            prepared_bytes = tri.cl_ring_bytes;                                                         \
        }                                                                                               \
        SSG_CUDA(cudaLaunchKernelEx(&cfg, kern, tri.nlev, lp, pm, pr, cd, val, rhs, aux, D, out, out2, dinv, st, \
                                    ring_cap));                                                         \
    } while (0)
    switch (mode) {
        case SW_FWD_DIV: SSG_CL(SW_FWD_DIV); break;
        case SW_BWD_IC: SSG_CL(SW_BWD_IC); break;
        case SW_BWD_DIV: SSG_CL(SW_BWD_DIV); break;
        default: SSG_CL(SW_FWD_EIS); break;
    }
#undef SSG_CL
}

template <typename T>
void sweep_cluster(const Tri &tri, const T *val, int mode, const T *rhs, const T *aux, const T *D, T *out, T *out2,
                   const T *dinv, const KState *st, int group, cudaStream_t s) {
    if (tri.n == 0) return;
    const int G = group ? group : sweep_group(tri);
    if (G == 8)
        launch_cluster<T, 8>(tri, val, mode, rhs, aux, D, out, out2, dinv, st, s);
    else if (G == 32)
        launch_cluster<T, 32>(tri, val, mode, rhs, aux, D, out, out2, dinv, st, s);
    else if (G == 4)
        launch_cluster<T, 4>(tri, val, mode, rhs, aux, D, out, out2, dinv, st, s);
    else
        launch_cluster<T, 16>(tri, val, mode, rhs, aux, D, out, out2, dinv, st, s);
    SSG_LAUNCHED();
}

int cluster_size_available() {
    if (g_cluster_size < 0) g_cluster_size = probe_cluster<double>(96 * 1024);
    return g_cluster_size;
}

#define SSG_INST(T)                                                                                              \
    template void sweep_cluster<T>(const Tri &, const T *, int, const T *, const T *, const T *, T *, T *,       \
                                   const T *, const KState *, int, cudaStream_t);
SSG_INST(double)
SSG_INST(cplx)
SSG_INST(float)
SSG_INST(cplxf)
#undef SSG_INST

}  // namespace ssg
