// ss_push_plan.cpp -- the push sweep's schedule (see ss_push.cu for the kernel).
//
// Partition: CTA c owns the c-th contiguous chunk of every level (rows in level
// order, then row id), as the lockstep cluster sweep does. Each row's
// off-diagonal entries are sorted by (dependency level, column); the entries of
// the level just before the row's are the row's "new" part, summed after the
// wait, the others its "old" part, summed a level early.
//
// Per entry of row t (level lt, owner c) reading row j (level lj, owner cj,
// production index oj within cj):
//   cj == c and slot oj % S_own not reused before the end of level lt: own ring;
//   cj != c and lt - lj <= LEAD + 1: the receive ring (j is pushed to c);
//   otherwise: the output vector in memory (cj == c: stored by this CTA at an
//   earlier step; cj != c: the producer's progress, acquired by the LEAD check,
//   covers the store).
// New entries must come from shared memory, else the plan is infeasible.
// Receive slots are assigned per consumer in (producer level, producer
// position) order around the ring; a slot is reused only by a value pushed at a
// level at least LEAD + 1 after the consumer's last read of the previous one, so
// the LEAD bound orders the read first.
#include "ss_push_plan.hpp"

#include <algorithm>
#include <cstdlib>
#include <exception>
#include <thread>

namespace ssg {

// The plan's row-, consumer- and record-wise passes run on host threads: each item's
// output has a place fixed before the pass (prefix sums), so the plan does not depend on
// the thread count. Two triangles are planned at once, so a plan takes half the cores;
// SSG_PLAN_THREADS (1-64) sets the count.
static int plan_threads() {
    if (const char *e = std::getenv("SSG_PLAN_THREADS")) {
        const int v = std::atoi(e);
        if (v >= 1 && v <= 64) return v;
    }
    const unsigned hc = std::thread::hardware_concurrency();
    return (int)std::max(1u, std::min(16u, hc / 2));
}
// f(begin, end) over [0, n) in nt contiguous parts; an exception in a part is rethrown here.
// A part whose thread cannot be started runs on the calling thread.
template <typename F>
static void par_for(int n, int nt, F f) {
    if (nt <= 1 || n < 4096) {
        f(0, n);
        return;
    }
    const int part = (n + nt - 1) / nt;
    std::vector<std::thread> pool;
    std::vector<std::exception_ptr> errs(nt);
    auto run = [&](int b, int e, int q) {
        try {
            f(b, e);
        } catch (...) {
            errs[q] = std::current_exception();
        }
    };
    std::vector<int> inline_parts;
    for (int q = 1; q < nt; ++q) {
        const int b = q * part, e = std::min(n, b + part);
        if (b >= e) break;
        try {
            pool.emplace_back(run, b, e, q);
        } catch (...) {
            inline_parts.push_back(q);
        }
    }
    run(0, std::min(n, part), 0);
    for (int q : inline_parts) run(q * part, std::min(n, q * part + part), q);
    for (auto &t : pool) t.join();
    for (auto &e : errs)
        if (e) std::rethrow_exception(e);
}

PushLayout push_layout(int S_own, int S_recv, int cap_rec, int elem, int NB) {
    PushLayout L{};
    L.S_own = S_own;
    L.S_recv = S_recv;
    L.R = PS_R;
    L.NB = NB;
    L.LEAD = PS_LEAD;
    L.cap_rec = cap_rec;
    int o = 0;
    L.o_x = o;
    o += ps_al16((S_own + S_recv) * elem);
    L.o_base = o;  // partial sums handed from the older-entry group to the newest-entry group, two levels
    o += ps_al16(2 * PS_MAXQ * PS_CT * elem);
    L.o_mbr = o;
    o += ps_al16(8 * L.R);
    L.o_mbs = o;
    o += ps_al16(8 * NB);
    L.o_prog = o;
    o += 16;
    L.o_tabring = o;  // two rings of 4 table entries (16 bytes each)
    o += 128;
    L.o_buf = o;
    o += NB * ps_al16(cap_rec);
    L.total = o;
    return L;
}

PushPlanHost push_plan_host(int n, int nlev, const int *lptr, const int *prp, const int *pci, const int *perm,
                            const int *level, const int *ipos, int C, int elem) {
    PushPlanHost P;
    auto fail = [&](const char *why) {
        P.ok = false;
        P.why = why;
        return P;
    };
    if (C <= 0 || n <= 0 || nlev < 2) return fail("no cluster, no rows or a single level");
    if (C > 64) return fail("cluster too large");
    const int LEAD = PS_LEAD;
    auto chunk_of = [&](int l, int c, int &rs, int &re) {
        const int L0 = lptr[l], L1 = lptr[l + 1];
        const int chunk = (L1 - L0 + C - 1) / C;
        rs = std::min(L0 + c * chunk, L1);
        re = std::min(rs + chunk, L1);
    };
    // partition and production order
    std::vector<unsigned char> owner(n);
    std::vector<int> ordc(n);
    std::vector<std::vector<int>> levof(C);  // level of each production index, per CTA
    int cap_r = 1;
    for (int l = 0; l < nlev; ++l)
        for (int c = 0; c < C; ++c) {
            int rs, re;
            chunk_of(l, c, rs, re);
            cap_r = std::max(cap_r, re - rs);
            for (int t = rs; t < re; ++t) {
                owner[t] = (unsigned char)c;
                ordc[t] = (int)levof[c].size();
                levof[c].push_back(l);
            }
        }
    if (cap_r > PS_CT * PS_MAXQ) return fail("a level chunk has more rows than the CTA holds");
    const int nt = plan_threads();
    // entries (off-diagonal) sorted per row by (dependency level, column); a failing row
    // is reported as the first in row order, whatever the thread count
    std::vector<int> sprp(n + 1, 0), nsp(n, 0), &vmap = P.vmap;
    par_for(n, nt, [&](int b, int e) {
        for (int t = b; t < e; ++t) {
            const int i = perm[t];
            int m = 0;
            for (int k = prp[t]; k < prp[t + 1]; ++k) m += pci[k] != i;
            sprp[t + 1] = m;
        }
    });
    for (int t = 0; t < n; ++t) sprp[t + 1] += sprp[t];
    vmap.assign((size_t)sprp[n], 0);
    std::vector<int> dep((size_t)sprp[n]);
    std::vector<int> bad_row(nt, n), bad_why(nt, 0);  // per part: first failing row, 1 not a dependency, 2 too long
    {
        const int part = (n + nt - 1) / nt;
        par_for(n, nt, [&](int b, int e) {
            const int q = n < 4096 ? 0 : b / part;
            std::vector<std::pair<long long, int>> row;  // (level << 32 | column, entry)
            for (int t = b; t < e; ++t) {
                const int i = perm[t], lt = level[i];
                row.clear();
                bool ok = true;
                for (int k = prp[t]; k < prp[t + 1]; ++k) {
                    const int j = pci[k];
                    if (j == i) continue;
                    if (j < 0 || j >= n || level[j] >= lt) {
                        ok = false;
                        break;
                    }
                    row.push_back({((long long)level[j] << 32) | (unsigned)j, k});
                }
                if (!ok || row.size() > 0xFFFF) {
                    bad_row[q] = t;
                    bad_why[q] = ok ? 2 : 1;
                    return;
                }
                std::sort(row.begin(), row.end());
                int nold = 0, o = sprp[t];
                for (auto &en : row) {
                    if ((int)(en.first >> 32) < lt - 1) ++nold;
                    vmap[o] = en.second;
                    dep[o] = (int)(en.first & 0xFFFFFFFF);
                    ++o;
                }
                nsp[t] = nold;
            }
        });
    }
    for (int q = 0; q < nt; ++q)
        if (bad_why[q]) return fail(bad_why[q] == 1 ? "an entry is not a dependency of its row"
                                                    : "a row longer than 65535 entries");
    {
        // (entry, row) of the newest entries, in row order: each row's place from a prefix sum
        std::vector<long long> nwp((size_t)n + 1, 0);
        for (int t = 0; t < n; ++t) nwp[t + 1] = nwp[t] + (sprp[t + 1] - sprp[t] - nsp[t]);
        P.dnew.assign((size_t)(2 * nwp[n]), 0);
        par_for(n, nt, [&](int b, int e) {
            for (int t = b; t < e; ++t) {
                size_t o = (size_t)(2 * nwp[t]);
                for (int k = sprp[t] + nsp[t]; k < sprp[t + 1]; ++k) {
                    P.dnew[o++] = k;
                    P.dnew[o++] = t;
                }
            }
        });
    }
    const int nent = (int)vmap.size();
    // codes; reads through the receive ring collected per consumer
    std::vector<int> code(nent, 0);
    struct Req {
        long long key;  // consumer << 58 | producer level << 32 | producer position
        int entry, use;
        bool operator<(const Req &o) const { return key < o.key || (key == o.key && entry < o.entry); }
    };
    // collected per part and consumer, then per consumer sorted: the key's top bits are the
    // consumer, so the consumers' sorted runs in order are the whole sorted list
    std::vector<std::vector<std::vector<Req>>> parts(nt, std::vector<std::vector<Req>>(C));
    {
        const int part = (n + nt - 1) / nt;
        par_for(n, nt, [&](int b, int e) {
            std::vector<std::vector<Req>> &mine = parts[n < 4096 ? 0 : b / part];
            for (int t = b; t < e; ++t) {
                const int c = owner[t], lt = level[perm[t]];
                for (int k = sprp[t]; k < sprp[t + 1]; ++k) {
                    const int j = dep[k], lj = level[j], pj = ipos[j], cj = owner[pj];
                    if (cj == c) {
                        continue;  // own ring or memory: depends on the ring size (per layout below)
                    } else if (lt - lj <= LEAD + 1) {
                        mine[c].push_back({((long long)c << 58) | ((long long)lj << 32) | (unsigned)pj, k, lt});
                    } else {
                        code[k] = j;
                    }
                }
            }
        });
    }
    std::vector<std::vector<Req>> byc(C);
    {
        std::vector<std::thread> pool;
        std::vector<std::exception_ptr> errs(C);
        auto one = [&](int c) {
            try {
                size_t total = 0;
                for (int q = 0; q < nt; ++q) total += parts[q][c].size();
                byc[c].reserve(total);
                for (int q = 0; q < nt; ++q) byc[c].insert(byc[c].end(), parts[q][c].begin(), parts[q][c].end());
                std::sort(byc[c].begin(), byc[c].end());
            } catch (...) {
                errs[c] = std::current_exception();
            }
        };
        for (int c0 = 0; c0 < C; c0 += nt) {  // at most nt consumers at a time
            std::vector<int> here{c0};        // consumers run on this thread
            for (int c = c0 + 1; c < std::min(C, c0 + nt); ++c) {
                try {
                    pool.emplace_back(one, c);
                } catch (...) {
                    here.push_back(c);
                }
            }
            for (int c : here) one(c);
            for (auto &t : pool) t.join();
            pool.clear();
        }
        for (auto &e : errs)
            if (e) std::rethrow_exception(e);
    }
    parts.clear();
    std::vector<Req> reqs;
    {
        size_t total = 0;
        for (int c = 0; c < C; ++c) total += byc[c].size();
        reqs.reserve(total);
        for (int c = 0; c < C; ++c) {
            reqs.insert(reqs.end(), byc[c].begin(), byc[c].end());
            std::vector<Req>().swap(byc[c]);
        }
    }
    struct Push {
        int c, pj, lp, last_use;
    };
    std::vector<Push> pushes;
    std::vector<int> pushof(reqs.size());
    for (size_t q = 0; q < reqs.size(); ++q) {
        const long long key = reqs[q].key;
        const int c = (int)(key >> 58), lp = (int)((key >> 32) & 0x3FFFFFF), pj = (int)(key & 0xFFFFFFFF);
        if (pushes.empty() || pushes.back().c != c || pushes.back().pj != pj) pushes.push_back({c, pj, lp, reqs[q].use});
        else pushes.back().last_use = std::max(pushes.back().last_use, reqs[q].use);
        pushof[q] = (int)pushes.size() - 1;
    }
    std::vector<int> pptr(n + 1, 0);
    for (auto &p : pushes) pptr[p.pj + 1]++;
    for (int t = 0; t < n; ++t) pptr[t + 1] += pptr[t];
    // records: per (pass, warp) slab widths; sizes; the largest
    std::vector<int> K;
    auto slab_widths = [&](int rs, int re) {
        const int cnt = re - rs;
        K.assign((size_t)ps_slots(cnt) / 32, 0);
        for (int q = 0; q < cnt; ++q) K[q / 32] = std::max(K[q / 32], sprp[rs + q + 1] - sprp[rs + q]);
        int ne = 0;
        for (int v : K) ne += 32 * v;
        return ne;
    };
    int cap_rec = 16, cnt_max = 0;
    for (int l = 0; l < nlev; ++l)
        for (int c = 0; c < C; ++c) {
            int rs, re;
            chunk_of(l, c, rs, re);
            const int ne = slab_widths(rs, re);
            const PsRec r = ps_rec(re - rs, ne, pptr[re] - pptr[rs], elem);
            cap_rec = std::max(cap_rec, r.size);
            cnt_max = std::max(cnt_max, re - rs);
        }
    // the layouts, largest rings and most staged records first: the ring sizes decide
    // which own entries stay in shared memory, the space left decides the receive ring
    // every attempt rewrites the code of each own-CTA entry (own ring or memory) and each
    // receive-ring entry; the entries read from memory across CTAs keep the code set above
    auto attempt = [&](int S_own, int NB) -> const char * {
        if (2 * cap_r > S_own) return "own ring smaller than two levels";
        PushLayout lay = push_layout(S_own, 0, cap_rec, elem, NB);
        // the receive ring takes the shared memory left next to the staged records
        int S_recv = std::min(1 << 16, (PS_SMEM_MAX - lay.total) / elem - 16);
        S_recv = (S_recv / 64) * 64;
        if (S_recv < 512) return ("no shared memory left for the receive ring");
        lay = push_layout(S_own, S_recv, cap_rec, elem, NB);
        if (lay.total > PS_SMEM_MAX) return ("layout exceeds shared memory");
        // own entries: the own ring while their slot is not reused before the end of the
        // reading row's level, else the output vector (never a newest entry)
        std::vector<char> left_ring(nt, 0);
        {
            const int part = (n + nt - 1) / nt;
            par_for(n, nt, [&](int b, int e) {
                char &flag = left_ring[n < 4096 ? 0 : b / part];
                for (int t = b; t < e && !flag; ++t) {
                    const int c = owner[t], lt = level[perm[t]];
                    for (int k = sprp[t]; k < sprp[t + 1]; ++k) {
                        const int j = dep[k], pj = ipos[j];
                        if (owner[pj] != c) continue;
                        const int oj = ordc[pj], reuse = oj + S_own;
                        const bool in_ring = reuse >= (int)levof[c].size() || levof[c][reuse] >= lt + 1;
                        if (in_ring) code[k] = -1 - (oj % S_own);
                        else if (level[j] != lt - 1) code[k] = j;
                        else flag = 1;
                    }
                }
            });
        }
        for (char f : left_ring)
            if (f) return "a newest own dependency left the own ring";
        // receive slots per consumer, and the reuse proof
        std::vector<int> slot(pushes.size());
        {
            std::vector<int> run(C, 0);
            std::vector<std::vector<int>> hist(C);
            for (size_t q = 0; q < pushes.size(); ++q) {
                const int c = pushes[q].c;
                const int k = run[c]++;
                slot[q] = k % S_recv;
                hist[c].push_back((int)q);
                if (k >= S_recv) {
                    const Push &old = pushes[hist[c][k - S_recv]];
                    if (old.last_use + 1 > pushes[q].lp - LEAD) return ("a receive slot is reused too early");
                }
            }
        }
        par_for((int)reqs.size(), nt, [&](int b, int e) {
            for (int q = b; q < e; ++q) code[reqs[q].entry] = -1 - (S_own + slot[pushof[q]]);
        });
        std::vector<int> plist(pushes.size());
        {
            std::vector<int> fillp(pptr.begin(), pptr.end() - 1);
            for (size_t q = 0; q < pushes.size(); ++q) plist[fillp[pushes[q].pj]++] = (pushes[q].c << 24) | slot[q];
        }
        std::vector<long long> bin((size_t)nlev * C, 0);
        for (auto &p : pushes) bin[(size_t)p.lp * C + p.c] += elem;
        // the records, in (level, CTA) order: sizes and offsets first (with the checks, in
        // record order), then every record filled on its own
        std::vector<int> &tab = P.tab, &rec = P.rec, &dval = P.dval, &dlv = P.dlv, &drhs = P.drhs;
        const int nrec = nlev * C;
        std::vector<long long> roff((size_t)nrec + 1, 0);
        std::vector<int> rne(nrec);
        for (int l = 0; l < nlev; ++l)
            for (int c = 0; c < C; ++c) {
                int rs, re;
                chunk_of(l, c, rs, re);
                const size_t id = (size_t)l * C + c;
                const int ne = slab_widths(rs, re);
                const PsRec r = ps_rec(re - rs, ne, pptr[re] - pptr[rs], elem);
                if (roff[id] + r.size >= (1ll << 31)) return ("records exceed 2 GB");
                if (bin[id] >= (1 << 20)) return ("a level pushes more bytes than a barrier counts");
                rne[id] = ne;
                roff[id + 1] = roff[id] + r.size;
            }
        tab.assign((size_t)nrec * 4, 0);
        rec.assign((size_t)(roff[nrec] / 4) + 16, 0);  // a copy never reads past the buffer
        dval.assign(nent, 0);
        dlv.assign(n, 0);
        drhs.assign(n, 0);
        par_for(nrec, nt, [&](int b, int e) {
            std::vector<int> Kl, slab;  // this part's slab widths and slab starts
            for (int id = b; id < e; ++id) {
                const int l = id / C, c = id % C;
                int rs, re;
                chunk_of(l, c, rs, re);
                const int cnt = re - rs, npass = 1, np = pptr[re] - pptr[rs];
                const int ne = rne[id];
                const PsRec r = ps_rec(cnt, ne, np, elem);
                const long long off = roff[id];
                Kl.assign((size_t)ps_slots(cnt) / 32, 0);
                for (int q = 0; q < cnt; ++q) Kl[q / 32] = std::max(Kl[q / 32], sprp[rs + q + 1] - sprp[rs + q]);
                int *tr = &tab[(size_t)id * 4];
                tr[0] = (int)(off / 16);
                tr[1] = r.size / 16;
                tr[2] = (int)bin[id];
                const size_t w0 = (size_t)(off / 4);
                rec[w0 + 0] = cnt;
                rec[w0 + 1] = ne;
                rec[w0 + 2] = np;
                bool hasg = false;  // an older entry read from the output vector (the kernel's slow path)
                for (int t = rs; t < re; ++t)
                    for (int k = sprp[t]; k < sprp[t + 1]; ++k) hasg = hasg || code[k] >= 0;
                rec[w0 + 3] = npass | ((hasg ? 1 : 0) << 16);
                const int slots = ps_slots(cnt);
                slab.assign(slots / 32, 0);  // first entry slot of each warp's slab
                for (int i = 0, acc = 0; i < slots / 32; ++i) {
                    slab[i] = acc;
                    acc += 32 * Kl[i];
                }
                int pnext = 0;
                for (int q = 0; q <= slots; ++q) {
                    int *ri = &rec[w0 + (r.o_info + 16 * q) / 4];
                    ri[3] = pnext;
                    if (q == slots || q >= cnt) {
                        ri[0] = q == slots ? ne : 0;
                        ri[1] = 0;
                        ri[2] = -1;
                        continue;
                    }
                    const int w = q / 32, lane = q % 32;
                    const int t = rs + q, e0 = sprp[t], len = sprp[t + 1] - e0;
                    const int first = slab[w] + lane;
                    ri[0] = first;
                    ri[1] = nsp[t] | (len << 16);
                    ri[2] = perm[t];
                    for (int k = 0; k < len; ++k) {
                        rec[w0 + r.o_code / 4 + first + 32 * k] = code[e0 + k];
                        dval[e0 + k] = (int)((off + r.o_val) / elem) + first + 32 * k;
                    }
                    for (int k = pptr[t]; k < pptr[t + 1]; ++k) rec[w0 + r.o_push / 4 + pnext++] = plist[k];
                    dlv[t] = (int)((off + r.o_lv) / elem) + q;
                    drhs[t] = (int)((off + r.o_rhs) / elem) + q;
                }
            }
        });
        P.C = C;
        P.nent = nent;
        P.npush = (int)pushes.size();
        P.cnt_max = cnt_max;
        P.lay = lay;
        P.ok = true;
        return nullptr;
    };
    const char *why = "no layout";
    for (int S_own : {PS_S_OWN, PS_S_OWN / 2, PS_S_OWN / 4, PS_S_OWN / 8})
        for (int NB = PS_NB; NB >= 3; --NB) {
            why = attempt(S_own, NB);
            if (!why) {
                P.ok = true;
                return P;
            }
        }
    return fail(why);
}

}  // namespace ssg
