/*
 * voxelgen.c -- seeded structured-voxel FEM systems for the Krylov hot path.
 *
 * Builds the systems the solvers are measured on: lowest-order edge
 * (Whitney / Nedelec first kind) elements on a uniform hexahedral voxel grid,
 *
 *   real     : K a = b               K_km = sum_e nu_e  int curl N_k . curl N_m
 *   complex  : (K + j omega M) a = b M_km = sum_e sig_e int N_k . N_m
 *
 * with the T-method source b_k = int N_k . curl T_h, where T_h is an edge
 * interpolant of a current vector potential supplied per z-directed edge.
 * curl T_h is divergence free by construction, so b is orthogonal to the
 * discrete gradients of interior nodal functions (the null space of K).
 *
 * The unknown ordering follows the reference example's mesh pipeline:
 *   - nodes are numbered breadth first from the origin, visiting the +x, +y,
 *     +z neighbours in that order
 *     (examples/VoxelFEM/MeshMakerFile/SearchTree.h:247-305);
 *   - edges are numbered per node in that order, x then y then z edge
 *     (MeshMakerFile/MeshMaker.h:170-244);
 *   - edges lying in a Dirichlet face (n x A = 0) are removed, the others are
 *     numbered consecutively in edge order (examples/VoxelFEM/VoxelMesh.cpp:297-319).
 * The element formulas are derived here from the basis functions and
 * integrated with 2x2x2 Gauss-Legendre points, which is exact for these
 * integrands (degree <= 2 per coordinate). The reference's closed forms
 * (examples/VoxelFEM/VoxelMatrix.cpp:118-201) are the same integrals.
 *
 * Duplicate (row, col) contributions are summed in element order; explicit
 * zeros stay in the pattern, as the reference's map-based builder keeps every
 * added position (src/SparseBuilder.cpp:107-141). Columns are sorted per row.
 *
 * Compile with -ffp-contract=off so that x86-64 and aarch64 builds produce
 * bit-identical matrices.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define VX_MAXROW 33 /* interior edge couples with 33 edges (itself included) */

typedef struct {
    int nx, ny, nz;           /* voxels per axis */
    double h;                 /* voxel edge length [m] */
    unsigned dirichlet_faces; /* bit 0:x=0 1:x=max 2:y=0 3:y=max 4:z=0 5:z=max */
    int order;                /* 0: breadth-first node order, 1: lexicographic */
} vx_grid;

static int64_t node_lin(const vx_grid *g, int x, int y, int z) {
    return (int64_t)x + (int64_t)(g->nx + 1) * ((int64_t)y + (int64_t)(g->ny + 1) * z);
}

/* node rank in the numbering order; rank[lin] */
static int build_node_rank(const vx_grid *g, int64_t *rank) {
    const int64_t nn = (int64_t)(g->nx + 1) * (g->ny + 1) * (g->nz + 1);
    if (g->order == 1) {
        for (int64_t i = 0; i < nn; ++i) rank[i] = i;
        return 0;
    }
    int64_t *queue = (int64_t *)malloc(sizeof(int64_t) * nn);
    unsigned char *seen = (unsigned char *)calloc(nn, 1);
    if (!queue || !seen) { free(queue); free(seen); return -1; }
    int64_t head = 0, tail = 0, id = 0;
    queue[tail++] = 0;
    seen[0] = 1;
    while (head < tail) {
        const int64_t v = queue[head++];
        rank[v] = id++;
        const int x = (int)(v % (g->nx + 1));
        const int y = (int)((v / (g->nx + 1)) % (g->ny + 1));
        const int z = (int)(v / ((int64_t)(g->nx + 1) * (g->ny + 1)));
        const int nb[3][3] = {{x + 1, y, z}, {x, y + 1, z}, {x, y, z + 1}};
        const int lim[3] = {g->nx, g->ny, g->nz};
        const int cur[3] = {x, y, z};
        for (int d = 0; d < 3; ++d) {
            if (cur[d] == lim[d]) continue;
            const int64_t w = node_lin(g, nb[d][0], nb[d][1], nb[d][2]);
            if (!seen[w]) { seen[w] = 1; queue[tail++] = w; }
        }
    }
    free(queue);
    free(seen);
    return 0;
}

static int on_dirichlet(const vx_grid *g, int dir, int x, int y, int z) {
    const unsigned f = g->dirichlet_faces;
    /* an edge lies in a face when both of its transverse coordinates allow it */
    const int c[3] = {x, y, z};
    const int lim[3] = {g->nx, g->ny, g->nz};
    for (int a = 0; a < 3; ++a) {
        if (a == dir) continue;
        if (c[a] == 0 && (f & (1u << (2 * a)))) return 1;
        if (c[a] == lim[a] && (f & (1u << (2 * a + 1)))) return 1;
    }
    return 0;
}

/*
 * Unknown index of each edge, addressed by (direction, start node).
 * emap[d][lin(node)] = unknown id, or -1 (Dirichlet or no such edge).
 * Returns the number of unknowns.
 */
static int64_t build_edge_maps(const vx_grid *g, int32_t *ex, int32_t *ey, int32_t *ez) {
    const int64_t nn = (int64_t)(g->nx + 1) * (g->ny + 1) * (g->nz + 1);
    int64_t *rank = (int64_t *)malloc(sizeof(int64_t) * nn);
    int64_t *byrank = (int64_t *)malloc(sizeof(int64_t) * nn);
    if (!rank || !byrank || build_node_rank(g, rank)) { free(rank); free(byrank); return -1; }
    for (int64_t i = 0; i < nn; ++i) byrank[rank[i]] = i;
    int32_t *maps[3] = {ex, ey, ez};
    const int lim[3] = {g->nx, g->ny, g->nz};
    int64_t nunk = 0;
    for (int64_t r = 0; r < nn; ++r) {
        const int64_t v = byrank[r];
        const int x = (int)(v % (g->nx + 1));
        const int y = (int)((v / (g->nx + 1)) % (g->ny + 1));
        const int z = (int)(v / ((int64_t)(g->nx + 1) * (g->ny + 1)));
        const int c[3] = {x, y, z};
        for (int d = 0; d < 3; ++d) {
            maps[d][v] = -1;
            if (c[d] == lim[d]) continue;
            if (on_dirichlet(g, d, x, y, z)) continue;
            maps[d][v] = (int32_t)nunk++;
        }
    }
    free(rank);
    free(byrank);
    return nunk;
}

/* ---------------- reference element (all 12 local edges) ----------------
 * local edge l = 4*d + 2*b + a : direction d, transverse offsets a (first
 * transverse axis) and b (second transverse axis), sign s = 2*offset-1.
 * Transverse axes: x-edge (y,z), y-edge (x,z), z-edge (x,y).                */
static void basis(int l, const double xi[3], const double L[3], double N[3], double C[3]) {
    const int d = l / 4, a = l & 1, b = (l >> 1) & 1;
    const double sa = 2.0 * a - 1.0, sb = 2.0 * b - 1.0;
    const int t1 = (d == 0) ? 1 : 0;       /* first transverse axis */
    const int t2 = (d == 2) ? 1 : 2;       /* second transverse axis */
    const double f1 = 1.0 + sa * xi[t1];
    const double f2 = 1.0 + sb * xi[t2];
    const double c = 1.0 / (8.0 * L[d]);
    N[0] = N[1] = N[2] = 0.0;
    N[d] = c * f1 * f2;
    /* derivatives of the scalar coefficient w.r.t. physical coordinates */
    double g[3] = {0.0, 0.0, 0.0};
    g[t1] = c * sa * f2 / L[t1];
    g[t2] = c * sb * f1 / L[t2];
    /* curl(w e_d) = grad(w) x e_d */
    double e[3] = {0.0, 0.0, 0.0};
    e[d] = 1.0;
    C[0] = g[1] * e[2] - g[2] * e[1];
    C[1] = g[2] * e[0] - g[0] * e[2];
    C[2] = g[0] * e[1] - g[1] * e[0];
}

static void element_matrices(double h, double K0[12][12], double M0[12][12], double C0[12][12]) {
    const double L[3] = {0.5 * h, 0.5 * h, 0.5 * h};
    const double q = 1.0 / sqrt(3.0);
    const double jac = L[0] * L[1] * L[2];
    memset(K0, 0, sizeof(double) * 144);
    memset(M0, 0, sizeof(double) * 144);
    memset(C0, 0, sizeof(double) * 144);
    for (int p = 0; p < 8; ++p) {
        const double xi[3] = {(p & 1) ? q : -q, (p & 2) ? q : -q, (p & 4) ? q : -q};
        double N[12][3], C[12][3];
        for (int l = 0; l < 12; ++l) basis(l, xi, L, N[l], C[l]);
        for (int k = 0; k < 12; ++k)
            for (int m = 0; m < 12; ++m) {
                K0[k][m] += jac * (C[k][0] * C[m][0] + C[k][1] * C[m][1] + C[k][2] * C[m][2]);
                M0[k][m] += jac * (N[k][0] * N[m][0] + N[k][1] * N[m][1] + N[k][2] * N[m][2]);
                C0[k][m] += jac * (N[k][0] * C[m][0] + N[k][1] * C[m][1] + N[k][2] * C[m][2]);
            }
    }
}

/* global unknown ids of the 12 local edges of element (x,y,z) */
static void element_edges(const vx_grid *g, const int32_t *const maps[3], int x, int y, int z, int32_t ids[12]) {
    for (int l = 0; l < 12; ++l) {
        const int d = l / 4, a = l & 1, b = (l >> 1) & 1;
        int c[3] = {x, y, z};
        const int t1 = (d == 0) ? 1 : 0;
        const int t2 = (d == 2) ? 1 : 2;
        c[t1] += a;
        c[t2] += b;
        ids[l] = maps[d][node_lin(g, c[0], c[1], c[2])];
    }
}

/* ---------------- public entry points ---------------- */

/* reference element matrices for unit material, exported for tests */
void vx_element_matrices(double h, double *K0, double *M0, double *C0) {
    element_matrices(h, (double (*)[12])K0, (double (*)[12])M0, (double (*)[12])C0);
}

/* unknown index of every (direction, start node) edge; arrays of (nx+1)(ny+1)(nz+1) */
int64_t vx_edge_maps(const vx_grid *g, int32_t *ex, int32_t *ey, int32_t *ez) {
    return build_edge_maps(g, ex, ey, ez);
}

/*
 * Assemble the system.
 *   nu[ne], sig[ne]  : per element reluctivity and conductivity, element
 *                      index x + nx*(y + ny*z); sig may be NULL
 *   tz[(nx+1)(ny+1)nz]: line integral of T along the z-edge starting at node
 *                      (x,y,z), index x + (nx+1)*(y + (ny+1)*z); may be NULL
 *   omega            : angular frequency scaling the mass term
 * Outputs (caller allocated, sizes from vx_count): row_ptr[n+1], col[nnz],
 * val_re[nnz], val_im[nnz] (may be NULL), b[n] (may be NULL).
 * Returns nnz, or -1 on allocation failure.
 */
static int64_t assemble(const vx_grid *g, const double *nu, const double *sig, double omega,
                        const double *tz, int32_t *row_ptr, int32_t *col, double *val_re,
                        double *val_im, double *b, int64_t *n_out) {
    const int64_t nn = (int64_t)(g->nx + 1) * (g->ny + 1) * (g->nz + 1);
    int32_t *ex = (int32_t *)malloc(sizeof(int32_t) * nn);
    int32_t *ey = (int32_t *)malloc(sizeof(int32_t) * nn);
    int32_t *ez = (int32_t *)malloc(sizeof(int32_t) * nn);
    if (!ex || !ey || !ez) { free(ex); free(ey); free(ez); return -1; }
    const int64_t n = build_edge_maps(g, ex, ey, ez);
    if (n < 0) { free(ex); free(ey); free(ez); return -1; }
    *n_out = n;
    const int32_t *const maps[3] = {ex, ey, ez};
    int32_t *rc = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * VX_MAXROW);
    unsigned char *cnt = (unsigned char *)calloc((size_t)n, 1);
    double *rk = NULL, *rm = NULL;
    const int want_vals = (row_ptr != NULL);
    if (want_vals) {
        rk = (double *)calloc((size_t)n * VX_MAXROW, sizeof(double));
        rm = (double *)calloc((size_t)n * VX_MAXROW, sizeof(double));
    }
    if (!rc || !cnt || (want_vals && (!rk || !rm))) {
        free(ex); free(ey); free(ez); free(rc); free(cnt); free(rk); free(rm);
        return -1;
    }
    double K0[12][12], M0[12][12], C0[12][12];
    element_matrices(g->h, K0, M0, C0);
    if (b && want_vals) memset(b, 0, sizeof(double) * (size_t)n);
    for (int z = 0; z < g->nz; ++z)
        for (int y = 0; y < g->ny; ++y)
            for (int x = 0; x < g->nx; ++x) {
                const int64_t e = (int64_t)x + (int64_t)g->nx * ((int64_t)y + (int64_t)g->ny * z);
                int32_t ids[12];
                element_edges(g, maps, x, y, z, ids);
                const double nue = nu ? nu[e] : 1.0;
                const double se = sig ? sig[e] * omega : 0.0;
                for (int k = 0; k < 12; ++k) {
                    const int32_t r = ids[k];
                    if (r < 0) continue;
                    int32_t *rowc = rc + (size_t)r * VX_MAXROW;
                    for (int m = 0; m < 12; ++m) {
                        const int32_t c = ids[m];
                        if (c < 0) continue;
                        int pos = -1;
                        for (int t = 0; t < cnt[r]; ++t)
                            if (rowc[t] == c) { pos = t; break; }
                        if (pos < 0) { pos = cnt[r]++; rowc[pos] = c; }
                        if (want_vals) {
                            rk[(size_t)r * VX_MAXROW + pos] += nue * K0[k][m];
                            rm[(size_t)r * VX_MAXROW + pos] += se * M0[k][m];
                        }
                    }
                    if (b && want_vals && tz) {
                        /* only z-directed local edges (8..11) carry T */
                        double acc = 0.0;
                        for (int m = 8; m < 12; ++m) {
                            const int a = m & 1, bb = (m >> 1) & 1;
                            const double t = tz[(int64_t)(x + a) + (int64_t)(g->nx + 1) * ((int64_t)(y + bb) + (int64_t)(g->ny + 1) * z)];
                            if (t != 0.0) acc += C0[k][m] * t;
                        }
                        b[r] += acc;
                    }
                }
            }
    /* sort each row by column and emit CSR */
    int64_t nnz = 0;
    for (int64_t r = 0; r < n; ++r) {
        int32_t *rowc = rc + (size_t)r * VX_MAXROW;
        double *rowk = want_vals ? rk + (size_t)r * VX_MAXROW : NULL;
        double *rowm = want_vals ? rm + (size_t)r * VX_MAXROW : NULL;
        const int c = cnt[r];
        for (int i = 1; i < c; ++i) {
            const int32_t kc = rowc[i];
            const double kk = want_vals ? rowk[i] : 0.0, km = want_vals ? rowm[i] : 0.0;
            int j = i - 1;
            while (j >= 0 && rowc[j] > kc) {
                rowc[j + 1] = rowc[j];
                if (want_vals) { rowk[j + 1] = rowk[j]; rowm[j + 1] = rowm[j]; }
                --j;
            }
            rowc[j + 1] = kc;
            if (want_vals) { rowk[j + 1] = kk; rowm[j + 1] = km; }
        }
        if (want_vals) {
            row_ptr[r] = (int32_t)nnz;
            for (int i = 0; i < c; ++i) {
                col[nnz + i] = rowc[i];
                val_re[nnz + i] = rowk[i];
                if (val_im) val_im[nnz + i] = rowm[i];
            }
        }
        nnz += c;
    }
    if (want_vals) row_ptr[n] = (int32_t)nnz;
    free(ex); free(ey); free(ez); free(rc); free(cnt); free(rk); free(rm);
    return nnz;
}

/* sizes of the system: returns nnz (>= 0) and writes n, or -1 on failure */
int64_t vx_count(const vx_grid *g, int64_t *n) {
    return assemble(g, NULL, NULL, 0.0, NULL, NULL, NULL, NULL, NULL, NULL, n);
}

/* right-hand side only: b[n] = sum_e C_e T_e for the given z-edge T values */
int64_t vx_rhs(const vx_grid *g, const double *tz, double *b) {
    const int64_t nn = (int64_t)(g->nx + 1) * (g->ny + 1) * (g->nz + 1);
    int32_t *ex = (int32_t *)malloc(sizeof(int32_t) * nn);
    int32_t *ey = (int32_t *)malloc(sizeof(int32_t) * nn);
    int32_t *ez = (int32_t *)malloc(sizeof(int32_t) * nn);
    if (!ex || !ey || !ez) { free(ex); free(ey); free(ez); return -1; }
    const int64_t n = build_edge_maps(g, ex, ey, ez);
    const int32_t *const maps[3] = {ex, ey, ez};
    double K0[12][12], M0[12][12], C0[12][12];
    element_matrices(g->h, K0, M0, C0);
    memset(b, 0, sizeof(double) * (size_t)n);
    for (int z = 0; z < g->nz; ++z)
        for (int y = 0; y < g->ny; ++y)
            for (int x = 0; x < g->nx; ++x) {
                int32_t ids[12];
                element_edges(g, maps, x, y, z, ids);
                for (int k = 0; k < 12; ++k) {
                    if (ids[k] < 0) continue;
                    double acc = 0.0;
                    for (int m = 8; m < 12; ++m) {
                        const int a = m & 1, bb = (m >> 1) & 1;
                        const double t = tz[(int64_t)(x + a) + (int64_t)(g->nx + 1) * ((int64_t)(y + bb) + (int64_t)(g->ny + 1) * z)];
                        if (t != 0.0) acc += C0[k][m] * t;
                    }
                    b[ids[k]] += acc;
                }
            }
    free(ex); free(ey); free(ez);
    return n;
}

int64_t vx_assemble(const vx_grid *g, const double *nu, const double *sig, double omega,
                    const double *tz, int32_t *row_ptr, int32_t *col, double *val_re,
                    double *val_im, double *b) {
    int64_t n = 0;
    return assemble(g, nu, sig, omega, tz, row_ptr, col, val_re, val_im, b, &n);
}
