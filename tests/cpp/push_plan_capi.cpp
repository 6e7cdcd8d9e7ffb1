// C entry points over the push sweep's host plan (ss_push_plan.cpp), for the
// CPU test that checks and emulates the schedule (tests/test_push_plan.py).
#include <cstring>

#include "ss_push_plan.hpp"

using ssg::PushPlanHost;

extern "C" {

void *pp_plan(int n, int nlev, const int *lptr, const int *prp, const int *pci, const int *perm, const int *level,
              const int *ipos, int C, int elem) {
    return new PushPlanHost(ssg::push_plan_host(n, nlev, lptr, prp, pci, perm, level, ipos, C, elem));
}

// info: ok, C, nent, npush, cnt_max, then the layout's ints in declaration order
int pp_info(void *h, int *info, int cap) {
    const PushPlanHost *P = (const PushPlanHost *)h;
    int v[5 + sizeof(ssg::PushLayout) / sizeof(int)];
    v[0] = P->ok;
    v[1] = P->C;
    v[2] = P->nent;
    v[3] = P->npush;
    v[4] = P->cnt_max;
    std::memcpy(v + 5, &P->lay, sizeof(ssg::PushLayout));
    const int m = (int)(sizeof(v) / sizeof(int));
    for (int i = 0; i < m && i < cap; ++i) info[i] = v[i];
    return m;
}

const char *pp_why(void *h) { return ((const PushPlanHost *)h)->why; }

// which: 0 tab, 1 rec, 2 vmap, 3 dval, 4 dlv, 5 drhs, 6 dnew; returns the length
int pp_get(void *h, int which, int *dst) {
    const PushPlanHost *P = (const PushPlanHost *)h;
    const std::vector<int> *a[] = {&P->tab, &P->rec, &P->vmap, &P->dval, &P->dlv, &P->drhs, &P->dnew};
    if (which < 0 || which > 6) return -1;
    if (dst && !a[which]->empty()) std::memcpy(dst, a[which]->data(), sizeof(int) * a[which]->size());
    return (int)a[which]->size();
}

void pp_free(void *h) { delete (PushPlanHost *)h; }

int pp_consts(int *out) {
    out[0] = ssg::PS_CT;
    out[1] = ssg::PS_MAXQ;
    out[2] = ssg::PS_SMEM_MAX;
    out[3] = ssg::PS_LEAD;
    out[4] = ssg::PS_NB;
    out[5] = ssg::PS_S_OWN;
    out[6] = ssg::PS_R;
    return 7;
}

// record section offsets for (rows, entry slots, pushes, elem): info, code, push, val, lv, rhs, size
void pp_rec(int cnt, int ne, int np, int elem, int *out) {
    const ssg::PsRec r = ssg::ps_rec(cnt, ne, np, elem);
    out[0] = r.o_info;
    out[1] = r.o_code;
    out[2] = r.o_push;
    out[3] = r.o_val;
    out[4] = r.o_lv;
    out[5] = r.o_rhs;
    out[6] = r.size;
}
}
