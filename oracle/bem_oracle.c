/* bem_oracle.c -- CPU ORACLE (test infrastructure, not the product).
 *
 * A plain-C restatement of the reference's geometry and panel quadrature
 * (squirmer-bem-3dtube, src/utils/{mesh,quadrature,kernels,field}.hpp), used
 * by oracle/oracle.py to check the CUDA path.  Only tests/, the smoke check and
 * bench.py's CPU-baseline leg load it.  Pinned against fixtures written by the
 * reference itself (tests/golden/, see tests/test_oracle.py).
 *
 * Everything is FP64 and follows the reference's evaluation order so the
 * results agree to the last bit where the compiler does not contract FMAs
 * (built with -ffp-contract=off).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846
#define ORC_8PI (8.0 * ORC_PI)

typedef struct { double x, y, z; } v3;
static v3 v_add(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static v3 v_sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static v3 v_scale(double s, v3 a) { v3 r = {s * a.x, s * a.y, s * a.z}; return r; }
static double v_dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 v_cross(v3 a, v3 b) {
    v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}
static double v_norm(v3 a) { return sqrt(v_dot(a, a)); }
static v3 v_unit(v3 a) { return v_scale(1.0 / v_norm(a), a); }
static v3 v_ld(const double* p) { v3 r = {p[0], p[1], p[2]}; return r; }
static void v_st(double* p, v3 a) { p[0] = a.x; p[1] = a.y; p[2] = a.z; }

/* ------------------------------------------------------------------ rules
 * quadrature.hpp:22-30 (Dunavant 7), 37-64 (subdivision), 69-72 (table),
 * 79-99 (Gauss-Legendre on [0, 1]). */
typedef struct { int n; double L[448][3]; double W[448]; } rule_t;
static rule_t g_rules[4];
static double g_gl_x[10], g_gl_w[10];
static int g_init = 0;

static void dunavant7(rule_t* r) {
    const double a1 = 0.059715871789770, b1 = 0.470142064105115, w1 = 0.132394152788506;
    const double a2 = 0.797426985353087, b2 = 0.101286507323456, w2 = 0.125939180544827;
    const double L[7][3] = {{1. / 3, 1. / 3, 1. / 3}, {a1, b1, b1}, {b1, a1, b1}, {b1, b1, a1},
                            {a2, b2, b2}, {b2, a2, b2}, {b2, b2, a2}};
    const double W[7] = {0.225, w1, w1, w1, w2, w2, w2};
    r->n = 7;
    memcpy(r->L, L, sizeof L);
    memcpy(r->W, W, sizeof W);
}

typedef struct { double p[3][3]; } tri3;

static void subdivided(int level, rule_t* out) {
    static tri3 a[64], b[64];
    int n = 1;
    memset(&a[0], 0, sizeof(tri3));
    a[0].p[0][0] = 1; a[0].p[1][1] = 1; a[0].p[2][2] = 1;
    for (int l = 0; l < level; ++l) {
        int m = 0;
        for (int t = 0; t < n; ++t) {
            double ab[3], bc[3], ca[3];
            for (int c = 0; c < 3; ++c) {
                ab[c] = (a[t].p[0][c] + a[t].p[1][c]) / 2;
                bc[c] = (a[t].p[1][c] + a[t].p[2][c]) / 2;
                ca[c] = (a[t].p[2][c] + a[t].p[0][c]) / 2;
            }
            for (int c = 0; c < 3; ++c) {
                b[m].p[0][c] = a[t].p[0][c]; b[m].p[1][c] = ab[c]; b[m].p[2][c] = ca[c];
                b[m + 1].p[0][c] = ab[c]; b[m + 1].p[1][c] = a[t].p[1][c]; b[m + 1].p[2][c] = bc[c];
                b[m + 2].p[0][c] = ca[c]; b[m + 2].p[1][c] = bc[c]; b[m + 2].p[2][c] = a[t].p[2][c];
                b[m + 3].p[0][c] = ab[c]; b[m + 3].p[1][c] = bc[c]; b[m + 3].p[2][c] = ca[c];
            }
            m += 4;
        }
        n = m;
        memcpy(a, b, sizeof(tri3) * n);
    }
    rule_t d;
    dunavant7(&d);
    out->n = 0;
    for (int t = 0; t < n; ++t)
        for (int q = 0; q < 7; ++q) {
            double l[3] = {0, 0, 0};
            for (int k = 0; k < 3; ++k)
                for (int c = 0; c < 3; ++c) l[c] += d.L[q][k] * a[t].p[k][c];
            memcpy(out->L[out->n], l, sizeof l);
            out->W[out->n] = d.W[q] / n;
            out->n++;
        }
}

static void gauss_legendre01(int n, double* x, double* w) {
    for (int i = 0; i < n; ++i) {
        double z = cos(ORC_PI * (i + 0.75) / (n + 0.5)), pp = 0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1, p2 = 0;
            for (int j = 1; j <= n; ++j) {
                double p3 = p2;
                p2 = p1;
                p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1);
            double dz = p1 / pp;
            z -= dz;
            if (fabs(dz) < 1e-15) break;
        }
        x[i] = 0.5 * (1 - z);
        w[i] = 1.0 / ((1 - z * z) * pp * pp);
    }
}

static void init_rules(void) {
    if (g_init) return;
    dunavant7(&g_rules[0]);
    subdivided(1, &g_rules[1]);
    subdivided(2, &g_rules[2]);
    subdivided(3, &g_rules[3]);
    gauss_legendre01(10, g_gl_x, g_gl_w);
    g_init = 1;
}

int orc_rule(int level, double* L, double* W) {
    init_rules();
    const rule_t* r = &g_rules[level];
    for (int q = 0; q < r->n; ++q) {
        L[3 * q] = r->L[q][0]; L[3 * q + 1] = r->L[q][1]; L[3 * q + 2] = r->L[q][2];
        W[q] = r->W[q];
    }
    return r->n;
}

void orc_gauss_legendre01(int n, double* x, double* w) { gauss_legendre01(n, x, w); }

/* ------------------------------------------------------------------ kernels
 * kernels.hpp:29-40 (accum_kernels), 50-65 (self_single_layer), 67-82
 * (panel_integrals), 107-111 (squirmer_slip). */
static void accum_kernels(v3 r, double w, v3 m, double* SL, double* DL) {
    double r2 = v_dot(r, r), rn = sqrt(r2), ir = 1 / rn, ir3 = ir / r2;
    double c[3] = {r.x, r.y, r.z};
    double d = -6 * w * v_dot(r, m) * ir3 / r2, s = w * ir3;
    for (int i = 0; i < 3; ++i) {
        SL[4 * i] += w * ir;
        for (int j = 0; j < 3; ++j) {
            SL[3 * i + j] += s * c[i] * c[j];
            DL[3 * i + j] += d * c[i] * c[j];
        }
    }
}

static void self_single_layer(const double* V9, v3 x0, double* SL) {
    double dummy[9];
    v3 zero = {0, 0, 0};
    for (int k = 0; k < 9; ++k) SL[k] = 0;
    for (int e = 0; e < 3; ++e) {
        v3 e1 = v_sub(v_ld(V9 + 3 * e), x0), e2 = v_sub(v_ld(V9 + 3 * ((e + 1) % 3)), x0);
        double J = v_norm(v_cross(e1, e2));
        for (int a = 0; a < 10; ++a)
            for (int b = 0; b < 10; ++b) {
                double u = g_gl_x[a], v = g_gl_x[b];
                v3 r = v_scale(u, v_add(v_scale(1 - v, e1), v_scale(v, e2)));
                accum_kernels(r, g_gl_w[a] * g_gl_w[b] * u * J, zero, SL, dummy);
            }
    }
}

/* geometry of one panel, as Mesh::geometry (mesh.hpp:61-72) */
typedef struct { double V[9]; v3 n, c; double area, h; } panel_t;

static void panel_geom(const double* V9, panel_t* P) {
    memcpy(P->V, V9, 9 * sizeof(double));
    v3 a = v_ld(V9), b = v_ld(V9 + 3), c = v_ld(V9 + 6);
    v3 cr = v_cross(v_sub(b, a), v_sub(c, a));
    P->area = 0.5 * v_norm(cr);
    P->n = v_scale(1.0 / (2 * P->area), cr);
    P->c = v_scale(1.0 / 3, v_add(v_add(a, b), c));
    P->h = sqrt(2 * P->area);
}

static void panel_integrals(const panel_t* P, v3 x0, int self, double* SL, double* DL) {
    for (int k = 0; k < 9; ++k) SL[k] = DL[k] = 0;
    if (self) {
        self_single_layer(P->V, x0, SL);
        return;
    }
    double d = v_norm(v_sub(P->c, x0)) / P->h;
    int lev = d < 0.75 ? 3 : (d < 1.5 ? 2 : (d < 3.0 ? 1 : 0));
    const rule_t* R = &g_rules[lev];
    v3 V0 = v_ld(P->V), V1 = v_ld(P->V + 3), V2 = v_ld(P->V + 6);
    for (int q = 0; q < R->n; ++q) {
        v3 x = v_add(v_add(v_scale(R->L[q][0], V0), v_scale(R->L[q][1], V1)), v_scale(R->L[q][2], V2));
        accum_kernels(v_sub(x, x0), R->W[q] * P->area, P->n, SL, DL);
    }
}

/* panel_integrals for a list of (panel, target, self) triples */
void orc_panel_integrals(int n, const double* V9, const double* x0, const int* self, double* SL,
                         double* DL) {
    init_rules();
    for (int k = 0; k < n; ++k) {
        panel_t P;
        panel_geom(V9 + 9 * k, &P);
        panel_integrals(&P, v_ld(x0 + 3 * k), self[k], SL + 9 * k, DL + 9 * k);
    }
}

/* quadrature rule index panel_integrals picks (kernels.hpp:74-75); 4 = self */
int orc_rule_of(const double* V9, const double* x0, int self) {
    if (self) return 4;
    panel_t P;
    panel_geom(V9, &P);
    double d = v_norm(v_sub(P.c, v_ld(x0))) / P.h;
    return d < 0.75 ? 3 : (d < 1.5 ? 2 : (d < 3.0 ? 1 : 0));
}

/* One coupling block, as the loops of swimmer.hpp:52-57, 188-216 and
 * duct_flow.hpp:382-397: targets are the centroids of mesh T, sources the panels
 * of mesh S; the self integral is used where same_mesh and i == p.
 *   Sblk (3nT x 3nS, column-major, ld 3nT) = SL / (8 pi mu)       (may be NULL)
 *   Dblk (same layout)                      = -DL / (8 pi)          (may be NULL)
 *   DLsum (9 per target, row-major)        += sum_p DL             (may be NULL) */
void orc_block(int nT, const double* VT, int nS, const double* VS, int same_mesh, double mu,
               double* Sblk, double* Dblk, double* DLsum) {
    init_rules();
    panel_t* ps = (panel_t*)malloc(sizeof(panel_t) * (size_t)nS);
    for (int p = 0; p < nS; ++p) panel_geom(VS + 9 * p, &ps[p]);
    size_t ld = 3 * (size_t)nT;
    double SL[9], DL[9];
    for (int i = 0; i < nT; ++i) {
        panel_t t;
        panel_geom(VT + 9 * i, &t);
        for (int p = 0; p < nS; ++p) {
            panel_integrals(&ps[p], t.c, same_mesh && i == p, SL, DL);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    size_t idx = (3 * (size_t)i + a) + (3 * (size_t)p + b) * ld;
                    if (Sblk) Sblk[idx] = SL[3 * a + b] / (ORC_8PI * mu);
                    if (Dblk) Dblk[idx] = -DL[3 * a + b] / ORC_8PI;
                }
            if (DLsum)
                for (int k = 0; k < 9; ++k) DLsum[9 * i + k] += DL[k];
        }
    }
    free(ps);
}

/* field.hpp:18-34 velocity_at: representation formula at each point */
void orc_velocity_at(int P, const double* V, const double* u, const double* f, double mu, int npts,
                     const double* pts, double* out) {
    init_rules();
    panel_t* ps = (panel_t*)malloc(sizeof(panel_t) * (size_t)P);
    for (int p = 0; p < P; ++p) panel_geom(V + 9 * p, &ps[p]);
    double SL[9], DL[9];
    for (int n = 0; n < npts; ++n) {
        double s[3] = {0, 0, 0};
        for (int p = 0; p < P; ++p) {
            panel_integrals(&ps[p], v_ld(pts + 3 * n), 0, SL, DL);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    s[j] += SL[3 * i + j] * f[3 * p + i] / (ORC_8PI * mu) - DL[3 * i + j] * u[3 * p + i] / ORC_8PI;
        }
        out[3 * n] = s[0]; out[3 * n + 1] = s[1]; out[3 * n + 2] = s[2];
    }
    free(ps);
}

/* ------------------------------------------------------------------ meshes
 * mesh.hpp:50-103 (Mesh, geometry, orient, merge), 112-136 (axial nodes),
 * 149-197 (tube), 208-245 (icosphere).  A mesh here is nodes + triangles +
 * tags; the caller receives per-panel vertices V (9 doubles) and tags. */
typedef struct {
    int nn, nt, capn, capt;
    double* nodes; /* 3 per node */
    int* tris;     /* 3 per triangle */
    int* tags;
} mesh_t;

static void m_init(mesh_t* m) { memset(m, 0, sizeof *m); }
static void m_free(mesh_t* m) { free(m->nodes); free(m->tris); free(m->tags); m_init(m); }
static void m_node(mesh_t* m, double x, double y, double z) {
    if (m->nn == m->capn) { m->capn = m->capn ? 2 * m->capn : 64; m->nodes = realloc(m->nodes, sizeof(double) * 3 * m->capn); }
    m->nodes[3 * m->nn] = x; m->nodes[3 * m->nn + 1] = y; m->nodes[3 * m->nn + 2] = z;
    m->nn++;
}
static void m_tri(mesh_t* m, int a, int b, int c, int tag) {
    if (m->nt == m->capt) {
        m->capt = m->capt ? 2 * m->capt : 64;
        m->tris = realloc(m->tris, sizeof(int) * 3 * m->capt);
        m->tags = realloc(m->tags, sizeof(int) * m->capt);
    }
    m->tris[3 * m->nt] = a; m->tris[3 * m->nt + 1] = b; m->tris[3 * m->nt + 2] = c;
    m->tags[m->nt] = tag;
    m->nt++;
}
static void m_panel(const mesh_t* m, int p, double* V9) {
    for (int k = 0; k < 3; ++k) memcpy(V9 + 3 * k, m->nodes + 3 * m->tris[3 * p + k], 3 * sizeof(double));
}
/* orient: flip where normal . outward(centroid) < 0 (mesh.hpp:76-81) */
typedef v3 (*outward_fn)(v3 x, const double* arg);
static void m_orient(mesh_t* m, outward_fn f, const double* arg) {
    for (int p = 0; p < m->nt; ++p) {
        double V9[9];
        panel_t P;
        m_panel(m, p, V9);
        panel_geom(V9, &P);
        if (v_dot(P.n, f(P.c, arg)) < 0) {
            int t = m->tris[3 * p + 1];
            m->tris[3 * p + 1] = m->tris[3 * p + 2];
            m->tris[3 * p + 2] = t;
        }
    }
}
static void m_merge(mesh_t* a, const mesh_t* b) {
    int off = a->nn;
    for (int k = 0; k < b->nn; ++k) m_node(a, b->nodes[3 * k], b->nodes[3 * k + 1], b->nodes[3 * k + 2]);
    for (int t = 0; t < b->nt; ++t)
        m_tri(a, b->tris[3 * t] + off, b->tris[3 * t + 1] + off, b->tris[3 * t + 2] + off, b->tags[t]);
}
static int m_out(const mesh_t* m, double* V, int* tags, int cap) {
    if (V && cap >= m->nt)
        for (int p = 0; p < m->nt; ++p) {
            m_panel(m, p, V + 9 * p);
            if (tags) tags[p] = m->tags[p];
        }
    return m->nt;
}

static v3 out_radial(v3 x, const double* arg) { (void)arg; v3 r = {x.x, x.y, 0}; return r; }
static v3 out_axial(v3 x, const double* arg) { (void)x; v3 r = {0, 0, arg[0]}; return r; }
static v3 out_center(v3 x, const double* arg) { return v_sub(v_ld(arg), x); }

static void tube_cap(mesh_t* m, double z0, int tag, double sg, double Rp, double al, int nth, int nr) {
    m_node(m, 0, 0, z0);
    for (int k = 1; k <= nr; ++k)
        for (int i = 0; i < nth; ++i)
            m_node(m, Rp * k / nr * cos(i * al), Rp * k / nr * sin(i * al), z0);
#define RING(k, i) (1 + (k) * nth + ((i) % nth))
    for (int i = 0; i < nth; ++i) m_tri(m, 0, RING(0, i), RING(0, i + 1), tag);
    for (int k = 0; k < nr - 1; ++k)
        for (int i = 0; i < nth; ++i) {
            int a = RING(k, i), b = RING(k, i + 1), c = RING(k + 1, i + 1), d = RING(k + 1, i);
            m_tri(m, a, d, c, tag);
            m_tri(m, a, c, b, tag);
        }
#undef RING
    m_orient(m, out_axial, &sg);
}

static void tube_mesh(double R, const double* z, int nz1, int nth, int nr, mesh_t* out) {
    double al = 2 * ORC_PI / nth;
    double Rp = R * sqrt(al / sin(al));
    int nz = nz1 - 1;
    mesh_t wall, cin, cout;
    m_init(&wall); m_init(&cin); m_init(&cout);
    for (int i = 0; i < nth; ++i)
        for (int k = 0; k <= nz; ++k) m_node(&wall, Rp * cos(i * al), Rp * sin(i * al), z[k]);
#define ID(i, k) (((i) % nth) * (nz + 1) + (k))
    for (int i = 0; i < nth; ++i)
        for (int k = 0; k < nz; ++k) {
            int a = ID(i, k), b = ID(i + 1, k), c = ID(i + 1, k + 1), d = ID(i, k + 1);
            m_tri(&wall, a, b, c, 0);
            m_tri(&wall, a, c, d, 0);
        }
#undef ID
    m_orient(&wall, out_radial, NULL);
    tube_cap(&cin, z[0], 1, -1.0, Rp, al, nth, nr);
    tube_cap(&cout, z[nz], 2, 1.0, Rp, al, nth, nr);
    m_merge(&wall, &cin);
    m_merge(&wall, &cout);
    m_free(&cin); m_free(&cout);
    *out = wall;
}

/* mesh.hpp:112-116 */
int orc_uniform_z(double z0, double z1, int nz, double* z) {
    for (int k = 0; k <= nz; ++k) z[k] = z0 + (z1 - z0) * k / nz;
    return nz + 1;
}

/* mesh.hpp:122-136; returns the node count (z may be NULL to count) */
int orc_graded_z(double L, double dzmin, double dzmax, double core, double growth, double* z, int cap) {
    int nh = 1, caph = 64;
    double* half = malloc(sizeof(double) * caph);
    half[0] = 0.0;
    double dz = dzmin;
    while (half[nh - 1] < L / 2 - 1e-12) {
        if (half[nh - 1] >= core) dz = fmin(dz * growth, dzmax);
        if (nh == caph) { caph *= 2; half = realloc(half, sizeof(double) * caph); }
        half[nh] = fmin(half[nh - 1] + dz, L / 2);
        nh++;
    }
    if (nh > 2 && L / 2 - half[nh - 2] < 0.3 * dz) {
        half[nh - 2] = half[nh - 1];
        nh--;
    }
    int n = 2 * nh - 1;
    if (z && cap >= n) {
        int k = 0;
        for (int i = nh - 1; i >= 0; --i) z[k++] = -half[i];
        for (int i = 1; i < nh; ++i) z[k++] = half[i];
    }
    free(half);
    return n;
}

int orc_tube_mesh(double R, const double* z, int nz1, int nth, int nr, double* V, int* tags, int cap) {
    init_rules();
    mesh_t m;
    tube_mesh(R, z, nz1, nth, nr, &m);
    int n = m_out(&m, V, tags, cap);
    m_free(&m);
    return n;
}

/* mesh.hpp:194-197 */
int orc_swimmer_tube_mesh(double R, double L, double a, int nth, int nr, double* V, int* tags, int cap) {
    double h = 2 * ORC_PI * R / nth;
    int nz1 = orc_graded_z(L, 0.6 * h, 1.4 * h, a + 0.5 * R, 1.25, NULL, 0);
    double* z = malloc(sizeof(double) * nz1);
    orc_graded_z(L, 0.6 * h, 1.4 * h, a + 0.5 * R, 1.25, z, nz1);
    int n = orc_tube_mesh(R, z, nz1, nth, nr, V, tags, cap);
    free(z);
    return n;
}

/* mesh.hpp:208-245 */
int orc_icosphere(double a, int level, double cx, double cy, double cz, int tag, double* V, int* tags, int cap) {
    double t = (1 + sqrt(5.0)) / 2;
    const double v0[12][3] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                              {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    const int F0[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                           {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
                           {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    int nv = 12, nf = 20;
    int maxv = 12, maxf = 20;
    for (int l = 0; l < level; ++l) { maxf *= 4; }
    maxv = maxf / 2 + 2;
    v3* v = malloc(sizeof(v3) * maxv);
    int* F = malloc(sizeof(int) * 3 * maxf);
    int* G = malloc(sizeof(int) * 3 * maxf);
    for (int i = 0; i < 12; ++i) v[i] = v_unit(v_ld(v0[i]));
    memcpy(F, F0, sizeof F0);
    for (int l = 0; l < level; ++l) {
        /* midpoint cache keyed on (min, max): open-addressing hash */
        int hcap = 1;
        while (hcap < 4 * 3 * nf) hcap <<= 1;
        long long* hk = malloc(sizeof(long long) * hcap);
        int* hv = malloc(sizeof(int) * hcap);
        for (int k = 0; k < hcap; ++k) hk[k] = -1;
        int ng = 0;
        for (int f = 0; f < nf; ++f) {
            int fv[3] = {F[3 * f], F[3 * f + 1], F[3 * f + 2]}, mids[3];
            for (int e = 0; e < 3; ++e) {
                int i = fv[e], j = fv[(e + 1) % 3];
                long long key = (long long)(i < j ? i : j) * 1000003LL + (i < j ? j : i);
                unsigned long long hsh = (unsigned long long)key * 0x9E3779B97F4A7C15ULL;
                int slot = (int)(hsh >> 40) & (hcap - 1);
                while (hk[slot] != -1 && hk[slot] != key) slot = (slot + 1) & (hcap - 1);
                if (hk[slot] == key) {
                    mids[e] = hv[slot];
                } else {
                    v[nv] = v_unit(v_add(v[i], v[j]));
                    hk[slot] = key;
                    hv[slot] = nv;
                    mids[e] = nv++;
                }
            }
            int ab = mids[0], bc = mids[1], ca = mids[2];
            int nfv[4][3] = {{fv[0], ab, ca}, {fv[1], bc, ab}, {fv[2], ca, bc}, {ab, bc, ca}};
            memcpy(G + 3 * ng, nfv, sizeof nfv);
            ng += 4;
        }
        free(hk); free(hv);
        nf = ng;
        int* tmp = F; F = G; G = tmp;
    }
    double vol = 0;
    for (int f = 0; f < nf; ++f) vol += v_dot(v[F[3 * f]], v_cross(v[F[3 * f + 1]], v[F[3 * f + 2]]));
    double s = cbrt(4 * ORC_PI / 3 / (fabs(vol) / 6));
    mesh_t m;
    m_init(&m);
    v3 c = {cx, cy, cz};
    for (int i = 0; i < nv; ++i) {
        v3 x = v_add(c, v_scale(a * s, v[i]));
        m_node(&m, x.x, x.y, x.z);
    }
    for (int f = 0; f < nf; ++f) m_tri(&m, F[3 * f], F[3 * f + 1], F[3 * f + 2], tag);
    double carg[3] = {cx, cy, cz};
    m_orient(&m, out_center, carg);
    int n = m_out(&m, V, tags, cap);
    m_free(&m);
    free(v); free(F); free(G);
    return n;
}

/* Mesh::geometry per panel (mesh.hpp:61-72) */
void orc_geometry(int P, const double* V, double* normal, double* centroid, double* area, double* h) {
    for (int p = 0; p < P; ++p) {
        panel_t g;
        panel_geom(V + 9 * p, &g);
        if (normal) v_st(normal + 3 * p, g.n);
        if (centroid) v_st(centroid + 3 * p, g.c);
        if (area) area[p] = g.area;
        if (h) h[p] = g.h;
    }
}

/* kernels.hpp:107-111 squirmer_slip at each point */
void orc_squirmer_slip(int n, const double* x, const double* center, const double* e, double B1, double B2,
                       double* out) {
    v3 c = v_ld(center), ev = v_ld(e);
    for (int p = 0; p < n; ++p) {
        v3 rh = v_unit(v_sub(v_ld(x + 3 * p), c));
        double ct = v_dot(rh, ev);
        v_st(out + 3 * p, v_scale(B1 + B2 * ct, v_sub(v_scale(ct, rh), ev)));
    }
}
