// ss_push_plan.hpp -- the push sweep's schedule, computed on the host from a
// level-ordered triangle (plain C++: the sweep's launcher in ss_push.cu and a
// CPU test that emulates the schedule both compile it).
#pragma once

#include <vector>

#ifdef __CUDACC__
#define SSG_HD __host__ __device__
#else
#define SSG_HD
#endif

namespace ssg {

constexpr int PS_CT = 256;                  // threads of each compute group (one row each)
// two compute groups (the newest entries of level l; the older entries of level l+1)
// and one warp that stages records, arms barriers and watches progress
constexpr int PS_THREADS = 2 * PS_CT + 32;
constexpr int PS_MAXQ = 1;                  // rows a compute thread holds per level
constexpr int PS_SMEM_MAX = 220 * 1024;     // dynamic shared memory a CTA may use
constexpr int PS_LEAD = 16;                 // levels a CTA may run ahead of the slowest
constexpr int PS_R = PS_LEAD + 4;           // receive barriers (one per producer level, round robin)
constexpr int PS_NB = 5;                    // staged level records at most (staged NB - 1 levels ahead)
constexpr int PS_S_OWN = 4096;              // own-ring slots at most

SSG_HD inline int ps_al16(int x) { return (x + 15) & ~15; }

// One level's chunk of one CTA as a contiguous record (staged with one bulk copy).
// Row q of the chunk is held by thread q of each compute group (at most PS_CT rows,
// one pass): rows fill warps densely, because GB300's FP64 pipe costs a warp
// instruction whatever the number of active lanes, so the fewest warps do a level's
// FP64 work in the fewest instructions, and a wide chunk runs as more warps at once
// rather than as a second pass. Each warp's entries form a slab, entry k of lane's
// row at slab + 32 * k + lane (ELL order: a warp's reads of entry k are consecutive).
// The per-row sections hold slots = rows rounded up to whole warps.
// Byte offsets from the record's start, each section 16-byte aligned:
//   [0]       header: rows cnt, entry slots ne, pushes np, 1 | (some entry read from
//             memory) << 16
//   [16]      row info, slots int4 by row: {first entry slot, old | all entries << 16,
//             row id (-1: no row), first push}; a row's pushes run to the next row's
//             first push (one closing int4 after the last slot)
//   codes     ne ints: >= 0 the output vector's row, < 0 shared-memory slot -1 - code
//             (own ring [0, S_own), then the receive ring)
//   pushes    np ints: consumer << 24 | receive slot
//   vals      ne values
//   lv        slots values: 1 / L_ii (forward) or D_i (backward), by row
//   rhs       slots values: the right-hand side (forward) or aux (backward)
struct PsRec {
    int o_info, o_code, o_push, o_val, o_lv, o_rhs, size;
};
// row slots of a record: its rows rounded up to whole warps
SSG_HD inline int ps_slots(int cnt) { return (cnt + 31) & ~31; }
SSG_HD inline PsRec ps_rec(int cnt, int ne, int np, int elem) {
    PsRec r;
    const int slots = ps_slots(cnt);
    r.o_info = 16;
    r.o_code = r.o_info + 16 * (slots + 1);
    r.o_push = r.o_code + ps_al16(4 * ne);
    r.o_val = r.o_push + ps_al16(4 * np);
    r.o_lv = r.o_val + ps_al16(elem * ne);
    r.o_rhs = r.o_lv + ps_al16(elem * slots);
    r.size = r.o_rhs + ps_al16(elem * slots);
    return r;
}

// Shared-memory carve-up of the push sweep, identical on host and device.
struct PushLayout {
    int S_own, S_recv;            // ring slots: values this CTA produced, values other CTAs pushed to it
    int R, NB, LEAD;              // receive barriers, staged records, most levels a CTA runs ahead
    int cap_rec;                  // bytes of the largest record
    // byte offsets
    int o_x, o_base, o_mbr, o_mbs, o_prog, o_tabring, o_buf;
    int total;
};
PushLayout push_layout(int S_own, int S_recv, int cap_rec, int elem, int NB);

// Host result of the plan. tab: per (level, CTA) int4 {record offset / 16,
// record bytes / 16, bytes other CTAs push to this CTA at this level, 0}.
// rec: the records (static parts filled, values zero), as ints. Per sorted
// entry k: vmap[k] its index in the triangle's layout, dval[k] the element
// index of its value in rec (in units of the value size); per level-ordered
// row t: dlv[t], drhs[t] likewise. dnew: pairs (entry k, row t) of the newest
// entries (dependency level one below the row's), whose values the records
// hold pre-scaled: -(value * lvec[t]).
struct PushPlanHost {
    bool ok = false;
    const char *why = "";
    int C = 0, nent = 0, npush = 0, cnt_max = 0;
    PushLayout lay{};
    std::vector<int> tab, rec, vmap, dval, dlv, drhs, dnew;
};

// n rows in level order: lptr[nlev+1] level pointers, prp/pci the level-ordered
// rows (columns as row ids, the diagonal included), perm[t] row of position t,
// level[row], ipos[row] position of a row. C CTAs, elem bytes a value. Tries
// own rings of 4096 down to 512 slots and 5 down to 3 staged records; the
// first that fits.
PushPlanHost push_plan_host(int n, int nlev, const int *lptr, const int *prp, const int *pci, const int *perm,
                            const int *level, const int *ipos, int C, int elem);

}  // namespace ssg
