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

constexpr int PS_CT = 128;                  // threads of each compute group (one row each per pass)
// two compute groups (the newest entries of level l; the older entries of level l+1)
// and one warp that stages records, arms barriers and watches progress
constexpr int PS_THREADS = 2 * PS_CT + 32;
constexpr int PS_MAXQ = 2;                  // rows a compute thread holds per level
constexpr int PS_SMEM_MAX = 220 * 1024;     // dynamic shared memory a CTA may use
constexpr int PS_LEAD = 16;                 // levels a CTA may run ahead of the slowest
constexpr int PS_R = PS_LEAD + 4;           // receive barriers (one per producer level, round robin)
constexpr int PS_NB = 5;                    // staged level records at most (staged NB - 1 levels ahead)
constexpr int PS_S_OWN = 4096;              // own-ring slots at most

SSG_HD inline int ps_al16(int x) { return (x + 15) & ~15; }

// One level's chunk of one CTA as a contiguous record (staged with one bulk copy).
// A row's off-diagonal entries split into its newest entries (dependency level
// one below the row's, summed by the newest-entry group after the wait) and its
// older entries (summed a level early by the older-entry group).
//
// Newest entries: row q of the chunk is held by thread q % PS_CT in pass
// q / PS_CT (rows fill warps densely: GB300's FP64 pipe costs a warp
// instruction whatever the number of active lanes); each warp's newest entries
// form a slab, entry k of lane's row at slab + 32 * k + lane.
//
// Older entries: each row's older entries, in (dependency level, column)
// order, are cut into pieces of PS_PIECE from the row's end (the first piece
// may be shorter); a piece is summed into one partial, and the row adds its
// pieces' partials in order. The pieces depend on the row alone, so a row's
// arithmetic does not depend on what else shares its level (a system gives the
// same bits alone and in a batch). The chunk's pieces, in row order, are dealt
// to the PS_CT threads, npt consecutive pieces each; a thread sums up to four
// pieces at a time, entry position j = 0..3 outer, piece inner, so its FP64
// chain is at most four deep. Pieces are right-aligned (a piece of s entries
// at positions 4 - s .. 3), which puts the entries of dependency level two
// below the row (the last of the row) at the highest positions: the wait for
// them comes late. Entry j of thread t's q-th piece sits at
// (4 q + j) * PS_CT + t.
//
// Byte offsets from the record's start, each section 16-byte aligned:
//   [0]       header, 8 ints: rows cnt, newest entry slots ne, pushes np,
//             passes npass | (some older entry read from memory) << 16, older
//             entries W, pieces per thread npt, pieces nseg, 0
//   [32]      row info, npass * PS_CT int4 by row: {first newest slot, newest
//             entries, row id (-1: no row), first push}; a row's pushes run to
//             the next row's first push (one closing int4 after the last slot)
//   sbeg      npass * PS_CT + 1 ints: the first piece of each row
//   tinfo     PS_CT int4 by thread: {sizes of its pieces (2 bits each, size -
//             1), entries of dependency level two below the row (bit 4 q + j),
//             0, 0}
//   codes     ne + 4 npt * PS_CT ints (newest slab, then the older pieces): >= 0 the
//             output vector's row, < 0 shared-memory slot -1 - code (own ring
//             [0, S_own), then the receive ring)
//   pushes    np ints: consumer << 24 | receive slot
//   vals      ne + 4 npt * PS_CT values, as the codes
//   lv        npass * PS_CT values: 1 / L_ii (forward) or D_i (backward), by row
//   rhs       npass * PS_CT values: the right-hand side (forward) or aux (backward)
constexpr int PS_PIECE = 4;                 // older entries summed into one partial
constexpr int PS_NPT = 8;                   // pieces a thread holds per level at most
constexpr int PS_SEGMAX = PS_NPT * PS_CT;   // pieces of one record at most
struct PsRec {
    int o_info, o_sbeg, o_tinfo, o_code, o_push, o_val, o_lv, o_rhs, size;
};
SSG_HD inline PsRec ps_rec(int npass, int ne, int npt, int np, int elem) {
    PsRec r;
    const int slots = npass * PS_CT, nv = ne + PS_PIECE * npt * PS_CT;
    r.o_info = 32;
    r.o_sbeg = r.o_info + 16 * (slots + 1);
    r.o_tinfo = r.o_sbeg + ps_al16(4 * (slots + 1));
    r.o_code = r.o_tinfo + 16 * PS_CT;
    r.o_push = r.o_code + ps_al16(4 * nv);
    r.o_val = r.o_push + ps_al16(4 * np);
    r.o_lv = r.o_val + ps_al16(elem * nv);
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
    int o_x, o_base, o_tp, o_mbr, o_mbs, o_prog, o_tabring, o_buf;
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
