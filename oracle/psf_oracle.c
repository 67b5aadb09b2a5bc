/*
 * psf_oracle.c -- CPU oracle for PANSFEM2's SIMP topology-optimisation path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE: only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference leg load it, as the checker.
 *
 * A plain-C restatement of the reference's algorithm.  Each routine names the
 * reference routine it follows and keeps its floating-point operation order:
 * sums start from 0.0 and run in the reference's loop order, products are
 * evaluated left to right, std::max/std::min keep their tie behaviour.  Built
 * with -ffp-contract=off it reproduces the reference bit for bit on one host.
 * The one structural liberty: temporaries are allocated once per call instead
 * of once per operator, which makes this CPU path faster than the reference,
 * never slower.
 */
#include "psf_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 0;
void orc_set_threads(int n) { g_threads = n; }
int orc_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

static void *xmalloc(size_t n) {
    void *p = malloc(n ? n : 1);
    if (!p) { fprintf(stderr, "psf_oracle: out of memory (%zu bytes)\n", n); abort(); }
    return p;
}
static void *xcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s ? s : 1);
    if (!p) { fprintf(stderr, "psf_oracle: out of memory\n"); abort(); }
    return p;
}
void orc_free(void *p) { free(p); }

/* std::max(a, b) / std::min(a, b): return the first argument on ties */
static inline double smax(double a, double b) { return (a < b) ? b : a; }
static inline double smin(double a, double b) { return (b < a) ? b : a; }

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* ======================= mesh (SquareMesh.h:61-106) ======================= */
void orc_q4_nodes(double lx, double ly, int nx, int ny, double *xy) {
    for (int i = 0; i < nx + 1; i++)
        for (int j = 0; j < ny + 1; j++) {
            long n = (long)(ny + 1) * i + j;
            xy[2 * n + 0] = lx * (i / (double)nx);
            xy[2 * n + 1] = ly * (j / (double)ny);
        }
}

void orc_q4_elements(int nx, int ny, int *conn) {
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            long e = (long)ny * i + j;
            conn[4 * e + 0] = (ny + 1) * i + j;
            conn[4 * e + 1] = (ny + 1) * (i + 1) + j;
            conn[4 * e + 2] = (ny + 1) * (i + 1) + (j + 1);
            conn[4 * e + 3] = (ny + 1) * i + (j + 1);
        }
}

static inline long h8_node(int ny, int nz, int i, int j, int k) {
    return ((long)(ny + 1) * i + j) * (nz + 1) + k;
}

void orc_h8_nodes(double lx, double ly, double lz, int nx, int ny, int nz, double *xyz) {
    for (int i = 0; i < nx + 1; i++)
        for (int j = 0; j < ny + 1; j++)
            for (int k = 0; k < nz + 1; k++) {
                long n = h8_node(ny, nz, i, j, k);
                xyz[3 * n + 0] = lx * (i / (double)nx);
                xyz[3 * n + 1] = ly * (j / (double)ny);
                xyz[3 * n + 2] = lz * (k / (double)nz);
            }
}

/* node order of ShapeFunction8Cubic::Points (ShapeFunction.h:299) */
void orc_h8_elements(int nx, int ny, int nz, int *conn) {
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                long e = ((long)ny * i + j) * nz + k;
                int *c = conn + 8 * e;
                c[0] = (int)h8_node(ny, nz, i, j, k);
                c[1] = (int)h8_node(ny, nz, i + 1, j, k);
                c[2] = (int)h8_node(ny, nz, i + 1, j + 1, k);
                c[3] = (int)h8_node(ny, nz, i, j + 1, k);
                c[4] = (int)h8_node(ny, nz, i, j, k + 1);
                c[5] = (int)h8_node(ny, nz, i + 1, j, k + 1);
                c[6] = (int)h8_node(ny, nz, i + 1, j + 1, k + 1);
                c[7] = (int)h8_node(ny, nz, i, j + 1, k + 1);
            }
}

/* =========== numbering (BoundaryCondition.h:19-25, Assembling.h:175-186) =========== */
int orc_renumber(int nnodes, int ndof, const unsigned char *fixed, int *n2g) {
    int K = 0;
    for (long a = 0; a < (long)nnodes * ndof; a++) n2g[a] = fixed[a] ? -1 : K++;
    return K;
}

/* ======================= small dense helpers (Matrix.h) ======================= */
/* C(r x c) = A(r x k) * B(k x c), each entry summed from 0 in k order (Matrix.h:243-256) */
static void mm(const double *A, const double *B, double *C, int r, int k, int c) {
    for (int i = 0; i < r; i++)
        for (int j = 0; j < c; j++) {
            double v = 0.0;
            for (int q = 0; q < k; q++) v += A[i * k + q] * B[q * c + j];
            C[i * c + j] = v;
        }
}
static void transpose(const double *A, double *T, int r, int c) {
    for (int i = 0; i < c; i++)
        for (int j = 0; j < r; j++) T[i * r + j] = A[j * c + i];
}
/* Determinant 2x2 / 3x3 (Matrix.h:326-342) */
static double det2(const double *v) { return v[0] * v[3] - v[1] * v[2]; }
static double det3(const double *v) {
    return -v[8] * v[1] * v[3] - v[7] * v[5] * v[0] - v[2] * v[4] * v[6] + v[6] * v[1] * v[5] +
           v[7] * v[3] * v[2] + v[0] * v[4] * v[8];
}
/* Cofactor (Matrix.h:363-385): drop row ri and column cj */
static void cofactor(const double *A, int n, int ri, int cj, double *C) {
    int m = n - 1;
    for (int i = 0; i < m; i++)
        for (int j = 0; j < m; j++) {
            int si = i < ri ? i : i + 1;
            int sj = j < cj ? j : j + 1;
            C[i * m + j] = A[si * n + sj];
        }
}
/* Inverse (Matrix.h:346-360): pow(-1, i+j) * det(Cofactor(j, i)), then / det */
static void inverse(const double *A, int n, double *inv) {
    double cof[9];
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            cofactor(A, n, j, i, cof);
            double d = (n == 2) ? cof[0] : det2(cof);
            inv[i * n + j] = pow(-1.0, i + j) * d;
        }
    double det = (n == 2) ? det2(A) : det3(A);
    for (int k = 0; k < n * n; k++) inv[k] /= det;
}

/* Gauss4Square points (GaussIntegration.h:143-148); weights are all 1.0 */
static void gauss4(int g, double *r) {
    double a = 1.0 / sqrt(3.0);
    static const int sx[4] = {-1, 1, -1, 1}, sy[4] = {-1, -1, 1, 1};
    r[0] = sx[g] < 0 ? -a : a;
    r[1] = sy[g] < 0 ? -a : a;
}
/* Gauss8Cubic points (GaussIntegration.h:231-240) */
static void gauss8(int g, double *r) {
    double a = 1.0 / sqrt(3.0);
    static const int s[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    for (int k = 0; k < 3; k++) r[k] = s[g][k] < 0 ? -a : a;
}
/* ShapeFunction4Square::dNdr (ShapeFunction.h:186-191), 2 x 4 */
static void dndr_q4(const double *r, double *d) {
    d[0] = -0.25 * (1.0 - r[1]); d[1] = 0.25 * (1.0 - r[1]);
    d[2] = 0.25 * (1.0 + r[1]);  d[3] = -0.25 * (1.0 + r[1]);
    d[4] = -0.25 * (1.0 - r[0]); d[5] = -0.25 * (1.0 + r[0]);
    d[6] = 0.25 * (1.0 + r[0]);  d[7] = 0.25 * (1.0 - r[0]);
}
/* ShapeFunction8Cubic::dNdr (ShapeFunction.h:318-329), 3 x 8 */
static void dndr_h8(const double *r, double *d) {
    double *a = d, *b = d + 8, *c = d + 16;
    a[0] = -0.125 * (1.0 - r[1]) * (1.0 - r[2]); a[1] = 0.125 * (1.0 - r[1]) * (1.0 - r[2]);
    a[2] = 0.125 * (1.0 + r[1]) * (1.0 - r[2]);  a[3] = -0.125 * (1.0 + r[1]) * (1.0 - r[2]);
    a[4] = -0.125 * (1.0 - r[1]) * (1.0 + r[2]); a[5] = 0.125 * (1.0 - r[1]) * (1.0 + r[2]);
    a[6] = 0.125 * (1.0 + r[1]) * (1.0 + r[2]);  a[7] = -0.125 * (1.0 + r[1]) * (1.0 + r[2]);
    b[0] = -0.125 * (1.0 - r[2]) * (1.0 - r[0]); b[1] = -0.125 * (1.0 - r[2]) * (1.0 + r[0]);
    b[2] = 0.125 * (1.0 - r[2]) * (1.0 + r[0]);  b[3] = 0.125 * (1.0 - r[2]) * (1.0 - r[0]);
    b[4] = -0.125 * (1.0 + r[2]) * (1.0 - r[0]); b[5] = -0.125 * (1.0 + r[2]) * (1.0 + r[0]);
    b[6] = 0.125 * (1.0 + r[2]) * (1.0 + r[0]);  b[7] = 0.125 * (1.0 + r[2]) * (1.0 - r[0]);
    c[0] = -0.125 * (1.0 - r[0]) * (1.0 - r[1]); c[1] = -0.125 * (1.0 + r[0]) * (1.0 - r[1]);
    c[2] = -0.125 * (1.0 + r[0]) * (1.0 + r[1]); c[3] = -0.125 * (1.0 - r[0]) * (1.0 + r[1]);
    c[4] = 0.125 * (1.0 - r[0]) * (1.0 - r[1]);  c[5] = 0.125 * (1.0 + r[0]) * (1.0 - r[1]);
    c[6] = 0.125 * (1.0 + r[0]) * (1.0 + r[1]);  c[7] = 0.125 * (1.0 - r[0]) * (1.0 + r[1]);
}

/* ===================== element matrices ===================== */
/* PlaneStrain.h:20-58: Ke = sum_g B^T D B J t w0 w1, D scaled by E/((1-2V)(1+V)) */
void orc_ke_planestrain_q4(const double *X, double E, double V, double t, double *Ke) {
    double D[9] = {1.0 - V, V, 0.0, V, 1.0 - V, 0.0, 0.0, 0.0, 0.5 * (1.0 - 2.0 * V)};
    double sc = E / ((1.0 - 2.0 * V) * (1.0 + V));
    for (int k = 0; k < 9; k++) D[k] *= sc;
    memset(Ke, 0, 64 * sizeof(double));
    for (int g = 0; g < 4; g++) {
        double r[2], dN[8], dXdr[4], inv[4], dNdX[8], B[24], Bt[24], BtD[24], K[64];
        gauss4(g, r);
        dndr_q4(r, dN);
        mm(dN, X, dXdr, 2, 4, 2);
        double J = det2(dXdr);
        inverse(dXdr, 2, inv);
        mm(inv, dN, dNdX, 2, 2, 4);
        for (int n = 0; n < 4; n++) {
            B[0 * 8 + 2 * n] = dNdX[0 * 4 + n]; B[0 * 8 + 2 * n + 1] = 0.0;
            B[1 * 8 + 2 * n] = 0.0;             B[1 * 8 + 2 * n + 1] = dNdX[1 * 4 + n];
            B[2 * 8 + 2 * n] = dNdX[1 * 4 + n]; B[2 * 8 + 2 * n + 1] = dNdX[0 * 4 + n];
        }
        transpose(B, Bt, 3, 8);
        mm(Bt, D, BtD, 8, 3, 3);
        mm(BtD, B, K, 8, 3, 8);
        for (int k = 0; k < 64; k++) {
            double v = K[k] * J;
            v = v * t;
            v = v * 1.0;
            v = v * 1.0;
            Ke[k] += v;
        }
    }
}

/* PlaneStrain.h:20-58 with ShapeFunction3Triangle (ShapeFunction.h:87-117) and
 * Gauss1Triangle (GaussIntegration.h:64-81): one point (1/3, 1/3), weights 1/sqrt(2) each */
void orc_ke_planestrain_t3(const double *X, double E, double V, double t, double *Ke) {
    double D[9] = {1.0 - V, V, 0.0, V, 1.0 - V, 0.0, 0.0, 0.0, 0.5 * (1.0 - 2.0 * V)};
    double sc = E / ((1.0 - 2.0 * V) * (1.0 + V));
    for (int k = 0; k < 9; k++) D[k] *= sc;
    memset(Ke, 0, 36 * sizeof(double));
    const double dN[6] = {1.0, 0.0, -1.0, 0.0, 1.0, -1.0};
    const double w = 1.0 / sqrt(2.0);
    double dXdr[4], inv[4], dNdX[6], B[18], Bt[18], BtD[18], K[36];
    mm(dN, X, dXdr, 2, 3, 2);
    double J = det2(dXdr);
    inverse(dXdr, 2, inv);
    mm(inv, dN, dNdX, 2, 2, 3);
    for (int n = 0; n < 3; n++) {
        B[0 * 6 + 2 * n] = dNdX[0 * 3 + n]; B[0 * 6 + 2 * n + 1] = 0.0;
        B[1 * 6 + 2 * n] = 0.0;             B[1 * 6 + 2 * n + 1] = dNdX[1 * 3 + n];
        B[2 * 6 + 2 * n] = dNdX[1 * 3 + n]; B[2 * 6 + 2 * n + 1] = dNdX[0 * 3 + n];
    }
    transpose(B, Bt, 3, 6);
    mm(Bt, D, BtD, 6, 3, 3);
    mm(BtD, B, K, 6, 3, 6);
    for (int k = 0; k < 36; k++) {
        double v = K[k] * J;
        v = v * t;
        v = v * w;
        v = v * w;
        Ke[k] += v;
    }
}

/* HeatTransfer.h:19-43: Ke = sum_g B^T B J alpha t w0 w1, B = dXdr^-1 dNdr */
void orc_ke_heat_q4(const double *X, double alpha, double t, double *Ke) {
    memset(Ke, 0, 16 * sizeof(double));
    for (int g = 0; g < 4; g++) {
        double r[2], dN[8], dXdr[4], inv[4], B[8], Bt[8], K[16];
        gauss4(g, r);
        dndr_q4(r, dN);
        mm(dN, X, dXdr, 2, 4, 2);
        double J = det2(dXdr);
        inverse(dXdr, 2, inv);
        mm(inv, dN, B, 2, 2, 4);
        transpose(B, Bt, 2, 4);
        mm(Bt, B, K, 4, 2, 4);
        for (int k = 0; k < 16; k++) {
            double v = K[k] * J;
            v = v * alpha;
            v = v * t;
            v = v * 1.0;
            v = v * 1.0;
            Ke[k] += v;
        }
    }
}

/* Solid.h:20-64: Ke = sum_g B^T C B J w0 w1 w2, 6x6 Voigt C scaled by E/((1+V)(1-2V)) */
void orc_ke_solid_h8(const double *X, double E, double V, double *Ke) {
    double C[36];
    memset(C, 0, sizeof C);
    C[0 * 6 + 0] = 1.0 - V; C[0 * 6 + 1] = V;       C[0 * 6 + 2] = V;
    C[1 * 6 + 0] = V;       C[1 * 6 + 1] = 1.0 - V; C[1 * 6 + 2] = V;
    C[2 * 6 + 0] = V;       C[2 * 6 + 1] = V;       C[2 * 6 + 2] = 1.0 - V;
    C[3 * 6 + 3] = 0.5 * (1.0 - 2.0 * V);
    C[4 * 6 + 4] = 0.5 * (1.0 - 2.0 * V);
    C[5 * 6 + 5] = 0.5 * (1.0 - 2.0 * V);
    double sc = E / ((1.0 + V) * (1.0 - 2.0 * V));
    for (int k = 0; k < 36; k++) C[k] *= sc;
    memset(Ke, 0, 576 * sizeof(double));
    double *B = xmalloc(sizeof(double) * 144), *Bt = xmalloc(sizeof(double) * 144),
           *BtC = xmalloc(sizeof(double) * 144), *K = xmalloc(sizeof(double) * 576);
    for (int g = 0; g < 8; g++) {
        double r[3], dN[24], dXdr[9], inv[9], dNdX[24];
        gauss8(g, r);
        dndr_h8(r, dN);
        mm(dN, X, dXdr, 3, 8, 3);
        double J = det3(dXdr);
        inverse(dXdr, 3, inv);
        mm(inv, dN, dNdX, 3, 3, 8);
        memset(B, 0, sizeof(double) * 144);
        for (int n = 0; n < 8; n++) {
            double d0 = dNdX[0 * 8 + n], d1 = dNdX[1 * 8 + n], d2 = dNdX[2 * 8 + n];
            B[0 * 24 + 3 * n] = d0;
            B[1 * 24 + 3 * n + 1] = d1;
            B[2 * 24 + 3 * n + 2] = d2;
            B[3 * 24 + 3 * n] = d1; B[3 * 24 + 3 * n + 1] = d0;
            B[4 * 24 + 3 * n + 1] = d2; B[4 * 24 + 3 * n + 2] = d1;
            B[5 * 24 + 3 * n] = d2; B[5 * 24 + 3 * n + 2] = d0;
        }
        transpose(B, Bt, 6, 24);
        mm(Bt, C, BtC, 24, 6, 6);
        mm(BtC, B, K, 24, 6, 24);
        for (int k = 0; k < 576; k++) {
            double v = K[k] * J;
            v = v * 1.0;
            v = v * 1.0;
            v = v * 1.0;
            Ke[k] += v;
        }
    }
    free(B); free(Bt); free(BtC); free(K);
}

void orc_kind_shape(int kind, int *nen, int *ndof, int *dim) {
    switch (kind) {
    case ORC_Q4_PLANE_STRAIN: *nen = 4; *ndof = 2; *dim = 2; break;
    case ORC_Q4_HEAT: *nen = 4; *ndof = 1; *dim = 2; break;
    case ORC_T3_PLANE_STRAIN: *nen = 3; *ndof = 2; *dim = 2; break;
    default: *nen = 8; *ndof = 3; *dim = 3; break;
    }
}

void orc_ke(int kind, const double *X, double E, double V, double t, double *Ke) {
    if (kind == ORC_Q4_PLANE_STRAIN) orc_ke_planestrain_q4(X, E, V, t, Ke);
    else if (kind == ORC_Q4_HEAT) orc_ke_heat_q4(X, E, t, Ke);
    else if (kind == ORC_T3_PLANE_STRAIN) orc_ke_planestrain_t3(X, E, V, t, Ke);
    else orc_ke_solid_h8(X, E, V, Ke);
}

static void gather_X(int nen, int dim, const int *enodes, const double *coords, double *X) {
    for (int i = 0; i < nen; i++)
        for (int k = 0; k < dim; k++) X[i * dim + k] = coords[(long)enodes[i] * dim + k];
}

/* ===================== LILCSR + assembly ===================== */
typedef struct { int n, cap; int *col; double *val; } lil_row;

/* LILCSR::get (LILCSR.h:105-114): linear scan, 0 when absent */
static double lil_get(const lil_row *r, int c) {
    for (int k = 0; k < r->n; k++)
        if (r->col[k] == c) return r->val[k];
    return 0.0;
}
/* LILCSR::set (LILCSR.h:91-102): overwrite if present, else append */
static void lil_set(lil_row *r, int c, double v) {
    for (int k = 0; k < r->n; k++)
        if (r->col[k] == c) { r->val[k] = v; return; }
    if (r->n == r->cap) {
        r->cap = r->cap ? 2 * r->cap : 16;
        r->col = realloc(r->col, sizeof(int) * r->cap);
        r->val = realloc(r->val, sizeof(double) * r->cap);
        if (!r->col || !r->val) { fprintf(stderr, "psf_oracle: out of memory\n"); abort(); }
    }
    r->col[r->n] = c;
    r->val[r->n] = v;
    r->n++;
}

typedef struct { int col; double val; } colval;
static int cmp_colval(const void *a, const void *b) {
    int ca = ((const colval *)a)->col, cb = ((const colval *)b)->col;
    return (ca > cb) - (ca < cb);
}

/* PlaneStrainBodyForce (PlaneStrain.h:503-534), uniform f: Fe = sum_g B^T f J t w0 w1 */
void orc_body_force(int kind, const double *X, double fx, double fy, double t, double *Fe) {
    const int nen = kind == ORC_T3_PLANE_STRAIN ? 3 : 4, ng = kind == ORC_T3_PLANE_STRAIN ? 1 : 4;
    for (int k = 0; k < 2 * nen; k++) Fe[k] = 0.0;
    for (int g = 0; g < ng; g++) {
        double r[2], N[4], dN[8], J2[4], w0, w1;
        if (kind == ORC_T3_PLANE_STRAIN) {
            r[0] = 1.0 / 3.0; r[1] = 1.0 / 3.0;
            N[0] = r[0]; N[1] = r[1]; N[2] = 1.0 - r[0] - r[1];
            const double d[6] = {1.0, 0.0, -1.0, 0.0, 1.0, -1.0};
            for (int k = 0; k < 6; k++) dN[k] = d[k];
            w0 = w1 = 1.0 / sqrt(2.0);
        } else {
            gauss4(g, r);
            N[0] = 0.25 * (1.0 - r[0]) * (1.0 - r[1]);
            N[1] = 0.25 * (1.0 + r[0]) * (1.0 - r[1]);
            N[2] = 0.25 * (1.0 + r[0]) * (1.0 + r[1]);
            N[3] = 0.25 * (1.0 - r[0]) * (1.0 + r[1]);
            dndr_q4(r, dN);
            w0 = w1 = 1.0;
        }
        mm(dN, X, J2, 2, nen, 2);
        double J = det2(J2);
        for (int n = 0; n < nen; n++)
            for (int c = 0; c < 2; c++) {
                double b0 = c == 0 ? N[n] : 0.0, b1 = c == 0 ? 0.0 : N[n];
                double v = 0.0;
                v += b0 * fx;
                v += b1 * fy;
                v = v * J;
                v = v * t;
                v = v * w0;
                v = v * w1;
                Fe[2 * n + c] += v;
            }
    }
}

/* PlaneStrainSurfaceForce<ShapeFunction2Line, Gauss1Line> (PlaneStrain.h:421-452), uniform
 * traction on the edges (2 nodes each), assembled in edge order into the free dofs */
void orc_edge_loads(int nedge, const int *edges, const double *coords, double tx, double ty, double t,
                    const int *n2g, double *F) {
    for (int k = 0; k < nedge; k++) {
        double X[4];
        for (int q = 0; q < 2; q++)
            for (int d = 0; d < 2; d++) X[q * 2 + d] = coords[(long)edges[2 * k + q] * 2 + d];
        const double r = 0.0;
        const double N[2] = {0.5 * (1 - r), 0.5 * (1 + r)}, dN[2] = {-0.5, 0.5};
        double dd[2];
        mm(dN, X, dd, 1, 2, 2);
        double q2 = 0.0;
        q2 += dd[0] * dd[0];
        q2 += dd[1] * dd[1];
        const double dl = sqrt(q2);
        for (int n = 0; n < 2; n++)
            for (int c = 0; c < 2; c++) {
                double b0 = c == 0 ? N[n] : 0.0, b1 = c == 0 ? 0.0 : N[n];
                double v = 0.0;
                v += b0 * tx;
                v += b1 * ty;
                v = v * dl;
                v = v * t;
                v = v * 2.0;
                double fe = 0.0 + v;
                int I = n2g[(long)edges[2 * k + n] * 2 + c];
                if (I != -1) F[I] += fe;
            }
    }
}

int orc_assemble(int kind, int ne, const int *conn, const double *coords, const double *E_e,
                 double V, double t, const int *n2g, const double *ufixed, int N,
                 orc_csr *out, double *F) {
    return orc_assemble_body(kind, ne, conn, coords, E_e, V, t, n2g, ufixed, N, 0, 0.0, 0.0, out, F);
}

/* orc_assemble with the uniform body force assembled after each element's stiffness terms
 * (sample_planestrain.cpp:38-47) */
int orc_assemble_body(int kind, int ne, const int *conn, const double *coords, const double *E_e,
                      double V, double t, const int *n2g, const double *ufixed, int N, int body, double bfx,
                      double bfy, orc_csr *out, double *F) {
    int nen, ndof, dim;
    orc_kind_shape(kind, &nen, &ndof, &dim);
    int nk = nen * ndof;
    lil_row *rows = xcalloc((size_t)N, sizeof(lil_row));
    double *Ke = xmalloc(sizeof(double) * nk * nk);
    double X[24];
    /* element loop of sample_optimize_density_oc.cpp:122-128 + Assembling.h:46-66 */
    for (int e = 0; e < ne; e++) {
        const int *en = conn + (long)e * nen;
        gather_X(nen, dim, en, coords, X);
        orc_ke(kind, X, E_e[e], V, t, Ke);
        for (int i = 0; i < nen; i++)
            for (int a = 0; a < ndof; a++) {
                int I = n2g[(long)en[i] * ndof + a];
                if (I == -1) continue;
                int li = ndof * i + a;
                for (int j = 0; j < nen; j++)
                    for (int b = 0; b < ndof; b++) {
                        int J = n2g[(long)en[j] * ndof + b];
                        int lj = ndof * j + b;
                        if (J != -1) {
                            lil_set(&rows[I], J, lil_get(&rows[I], J) + Ke[li * nk + lj]);
                        } else {
                            double uf = ufixed ? ufixed[(long)en[j] * ndof + b] : 0.0;
                            F[I] -= Ke[li * nk + lj] * uf;
                        }
                    }
            }
        if (body) {
            double Fe[8];
            orc_body_force(kind, X, bfx, bfy, t, Fe);
            for (int i = 0; i < nen; i++)
                for (int a = 0; a < ndof; a++) {
                    int I = n2g[(long)en[i] * ndof + a];
                    if (I != -1) F[I] += Fe[ndof * i + a];
                }
        }
    }
    free(Ke);
    /* CSR(LILCSR&) (CSR.h:92-105): row sizes, per-row sort by column, concatenation */
    out->rows = N;
    out->indptr = xmalloc(sizeof(int) * ((size_t)N + 1));
    out->indptr[0] = 0;
    long long nnz = 0;
    for (int i = 0; i < N; i++) {
        nnz += rows[i].n;
        out->indptr[i + 1] = (int)nnz;
    }
    out->nnz = nnz;
    out->indices = xmalloc(sizeof(int) * (size_t)nnz);
    out->data = xmalloc(sizeof(double) * (size_t)nnz);
    colval *tmp = xmalloc(sizeof(colval) * 1024);
    int tcap = 1024;
    for (int i = 0; i < N; i++) {
        int n = rows[i].n;
        if (n > tcap) { tcap = n; tmp = realloc(tmp, sizeof(colval) * tcap); }
        for (int k = 0; k < n; k++) { tmp[k].col = rows[i].col[k]; tmp[k].val = rows[i].val[k]; }
        qsort(tmp, n, sizeof(colval), cmp_colval);
        long long o = out->indptr[i];
        for (int k = 0; k < n; k++) { out->indices[o + k] = tmp[k].col; out->data[o + k] = tmp[k].val; }
        free(rows[i].col);
        free(rows[i].val);
    }
    free(tmp);
    free(rows);
    return 0;
}

void orc_csr_free(orc_csr *A) {
    free(A->indptr); free(A->indices); free(A->data);
    A->indptr = NULL; A->indices = NULL; A->data = NULL;
}

/* Assembling(F, qfixed, nodetoglobal) (Assembling.h:151-158) */
void orc_neumann(int nload, const int *node, const int *dof, const double *val, int ndof,
                 const int *n2g, double *F) {
    for (int k = 0; k < nload; k++) {
        int I = n2g[(long)node[k] * ndof + dof[k]];
        if (I != -1) F[I] += val[k];
    }
}

/* ===================== linear algebra (CG.h) ===================== */
/* CSR::operator* (CSR.h:108-122): OpenMP over rows, each row summed in column order */
void orc_spmv(const orc_csr *A, const double *x, double *y) {
    int rows = A->rows;
    const int *ip = A->indptr, *ix = A->indices;
    const double *d = A->data;
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int i = 0; i < rows; i++) {
        double v = 0.0;
        for (int j = ip[i]; j < ip[i + 1]; j++) v += d[j] * x[ix[j]];
        y[i] = v;
    }
}

/* CSR::get (CSR.h:154-167): binary search (lower_bound) in the row */
double orc_csr_get(const orc_csr *A, int row, int col) {
    int lo = A->indptr[row], hi = A->indptr[row + 1];
    while (lo < hi) {
        int mid = lo + (hi - lo) / 2;
        if (A->indices[mid] < col) lo = mid + 1; else hi = mid;
    }
    if (lo == A->indptr[row + 1]) return 0.0;
    return A->indices[lo] == col ? A->data[lo] : 0.0;
}

/* CSR::set (CSR.h:125-151): overwrite if present, else insert keeping columns sorted */
int orc_csr_set(orc_csr *A, int row, int col, double v) {
    int lo = A->indptr[row], hi = A->indptr[row + 1];
    int end = hi;
    while (lo < hi) {
        int mid = lo + (hi - lo) / 2;
        if (A->indices[mid] < col) lo = mid + 1; else hi = mid;
    }
    if (lo != end && A->indices[lo] == col) { A->data[lo] = v; return 1; }
    A->nnz++;
    A->indices = realloc(A->indices, sizeof(int) * A->nnz);
    A->data = realloc(A->data, sizeof(double) * A->nnz);
    memmove(A->indices + lo + 1, A->indices + lo, sizeof(int) * (A->nnz - 1 - lo));
    memmove(A->data + lo + 1, A->data + lo, sizeof(double) * (A->nnz - 1 - lo));
    A->indices[lo] = col;
    A->data[lo] = v;
    for (int r = row + 1; r <= A->rows; r++) A->indptr[r]++;
    return 0;
}

/* std::inner_product with init 0: sequential left-to-right sum */
static double dot(const double *a, const double *b, long n) {
    double s = 0.0;
    for (long i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

/* ScalingCG (CG.h:419-453): Jacobi-preconditioned CG from x0 = 0, stop on the
 * recurrence residual ||r_k|| < eps*||b|| */
int orc_scaling_cg(const orc_csr *A, const double *b, int itmax, double eps, double *x) {
    long n = A->rows;
    double *D = xmalloc(sizeof(double) * n), *r = xmalloc(sizeof(double) * n),
           *p = xmalloc(sizeof(double) * n), *Mr = xmalloc(sizeof(double) * n),
           *Ap = xmalloc(sizeof(double) * n);
    for (long i = 0; i < n; i++) D[i] = orc_csr_get(A, (int)i, (int)i);      /* GetDiagonal :397-404 */
    for (long i = 0; i < n; i++) x[i] = 0.0;
    orc_spmv(A, x, Ap);
    for (long i = 0; i < n; i++) r[i] = b[i] - Ap[i];                         /* subtract :17-27 */
    for (long i = 0; i < n; i++) p[i] = r[i] / D[i];                          /* Scaling :408-415 */
    memcpy(Mr, p, sizeof(double) * n);
    double bnorm = sqrt(dot(b, b, n));
    double Mrr = dot(Mr, r, n);
    int ret = -1;
    for (int k = 0; k < itmax; ++k) {
        orc_spmv(A, p, Ap);
        double alpha = Mrr / dot(p, Ap, n);
        for (long i = 0; i < n; i++) x[i] = x[i] + alpha * p[i];             /* xexpay :31-38 */
        double malpha = -alpha;
        for (long i = 0; i < n; i++) r[i] = r[i] + malpha * Ap[i];
        for (long i = 0; i < n; i++) Mr[i] = r[i] / D[i];
        double Mrr1 = dot(Mr, r, n);
        double beta = Mrr1 / Mrr;
        for (long i = 0; i < n; i++) p[i] = beta * p[i] + Mr[i];              /* xeaxpy :42-49 */
        Mrr = Mrr1;
        double rnorm = sqrt(dot(r, r, n));
        if (rnorm < eps * bnorm) { ret = k + 1; break; }
    }
    free(D); free(r); free(p); free(Mr); free(Ap);
    return ret;
}

/* CG (CG.h:123-154) */
int orc_cg(const orc_csr *A, const double *b, int itmax, double eps, double *x) {
    long n = A->rows;
    double *r = xmalloc(sizeof(double) * n), *p = xmalloc(sizeof(double) * n),
           *Ap = xmalloc(sizeof(double) * n);
    for (long i = 0; i < n; i++) x[i] = 0.0;
    orc_spmv(A, x, Ap);
    for (long i = 0; i < n; i++) r[i] = b[i] - Ap[i];
    memcpy(p, r, sizeof(double) * n);
    double bnorm = sqrt(dot(b, b, n));
    double rr = dot(r, r, n);
    int ret = -1;
    for (int k = 0; k < itmax; ++k) {
        orc_spmv(A, p, Ap);
        double alpha = rr / dot(p, Ap, n);
        for (long i = 0; i < n; i++) x[i] = x[i] + alpha * p[i];
        double malpha = -alpha;
        for (long i = 0; i < n; i++) r[i] = r[i] + malpha * Ap[i];
        double rr1 = dot(r, r, n);
        double beta = rr1 / rr;
        for (long i = 0; i < n; i++) p[i] = beta * p[i] + r[i];
        rr = rr1;
        if (sqrt(rr) < eps * bnorm) { ret = k + 1; break; }
    }
    free(r); free(p); free(Ap);
    return ret;
}

/* BiCGSTAB (CG.h:158-193) */
int orc_bicgstab(const orc_csr *A, const double *b, int itmax, double eps, double *x) {
    long n = A->rows;
    double *r = xmalloc(sizeof(double) * n), *rd = xmalloc(sizeof(double) * n),
           *p = xmalloc(sizeof(double) * n), *Ap = xmalloc(sizeof(double) * n),
           *s = xmalloc(sizeof(double) * n), *As = xmalloc(sizeof(double) * n);
    for (long i = 0; i < n; i++) x[i] = 0.0;
    orc_spmv(A, x, Ap);
    for (long i = 0; i < n; i++) r[i] = b[i] - Ap[i];
    memcpy(rd, r, sizeof(double) * n);
    memcpy(p, r, sizeof(double) * n);
    double rdr = dot(rd, r, n);
    double bnorm = sqrt(dot(b, b, n));
    int ret = -1;
    for (int k = 0; k < itmax; ++k) {
        orc_spmv(A, p, Ap);
        double alpha = rdr / dot(rd, Ap, n);
        double malpha = -alpha;
        for (long i = 0; i < n; i++) s[i] = 1.0 * r[i] + malpha * Ap[i];   /* zeaxpby :79-88 */
        orc_spmv(A, s, As);
        double omega = dot(As, s, n) / dot(As, As, n);
        for (long i = 0; i < n; i++) x[i] = 1.0 * x[i] + alpha * p[i] + omega * s[i]; /* :67-74 */
        double momega = -omega;
        for (long i = 0; i < n; i++) r[i] = 1.0 * s[i] + momega * As[i];
        double rdr1 = dot(rd, r, n);
        double beta = alpha / omega * rdr1 / rdr;
        double mbo = -beta * omega;
        for (long i = 0; i < n; i++) p[i] = beta * p[i] + 1.0 * r[i] + mbo * Ap[i];
        rdr = rdr1;
        if (sqrt(dot(r, r, n)) < eps * bnorm) { ret = k + 1; break; }
    }
    free(r); free(rd); free(p); free(Ap); free(s); free(As);
    return ret;
}

/* BiCGSTAB2 (CG.h:197-253), the solver of src/LinearAlgebra/Solvers/test_CG.cpp */
int orc_bicgstab2(const orc_csr *A, const double *b, int itmax, double eps, double *x) {
    long n = A->rows;
    size_t sz = sizeof(double) * n;
    double *r = xmalloc(sz), *rd = xmalloc(sz), *p = xcalloc(n, 8), *u = xcalloc(n, 8),
           *tkm1 = xcalloc(n, 8), *w = xcalloc(n, 8), *z = xcalloc(n, 8), *Ap = xmalloc(sz),
           *y = xmalloc(sz), *tk = xmalloc(sz), *At = xmalloc(sz);
    for (long i = 0; i < n; i++) x[i] = 0.0;
    orc_spmv(A, x, Ap);
    for (long i = 0; i < n; i++) r[i] = b[i] - Ap[i];
    memcpy(rd, r, sz);
    double beta = 0.0;
    double rdr = dot(rd, r, n);
    double bnorm = sqrt(dot(b, b, n));
    int ret = -1;
    for (int k = 0; k < itmax; k++) {
        double mb = -beta;
        for (long i = 0; i < n; i++) p[i] = beta * p[i] + 1.0 * r[i] + mb * u[i];
        orc_spmv(A, p, Ap);
        double alpha = rdr / dot(rd, Ap, n);
        double ma = -alpha;
        for (long i = 0; i < n; i++)                                             /* :108-119 */
            y[i] = 1.0 * tkm1[i] + -1.0 * r[i] + ma * w[i] + alpha * Ap[i];
        for (long i = 0; i < n; i++) tk[i] = 1.0 * r[i] + ma * Ap[i];
        orc_spmv(A, tk, At);
        double Att = dot(At, tk, n), AtAt = dot(At, At, n), zeta, ita;
        if (k % 2 == 0) {
            zeta = Att / AtAt;
            ita = 0.0;
        } else {
            double yy = dot(y, y, n), yt = dot(y, tk, n), Aty = dot(At, y, n);
            zeta = (yy * Att - yt * Aty) / (AtAt * yy - Aty * Aty);
            ita = (AtAt * yt - Aty * Att) / (AtAt * yy - Aty * Aty);
        }
        for (long i = 0; i < n; i++)                                             /* :53-62 */
            u[i] = zeta * Ap[i] + ita * (tkm1[i] - r[i] + beta * u[i]);
        for (long i = 0; i < n; i++) z[i] = ita * z[i] + zeta * r[i] + ma * u[i];
        for (long i = 0; i < n; i++) x[i] = 1.0 * x[i] + alpha * p[i] + 1.0 * z[i];
        double mi = -ita, mz = -zeta;
        for (long i = 0; i < n; i++) r[i] = 1.0 * tk[i] + mi * y[i] + mz * At[i];
        double rdr1 = dot(rd, r, n);
        beta = alpha * rdr1 / (zeta * rdr);
        for (long i = 0; i < n; i++) w[i] = 1.0 * At[i] + beta * Ap[i];
        rdr = rdr1;
        memcpy(tkm1, tk, sz);
        if (sqrt(dot(r, r, n)) < eps * bnorm) { ret = k + 1; break; }
    }
    free(r); free(rd); free(p); free(u); free(tkm1); free(w); free(z); free(Ap); free(y);
    free(tk); free(At);
    return ret;
}

static int csr_has(const orc_csr *A, int row, int col) {
    int lo = A->indptr[row], hi = A->indptr[row + 1];
    while (lo < hi) {
        int mid = lo + (hi - lo) / 2;
        if (A->indices[mid] < col) lo = mid + 1; else hi = mid;
    }
    return lo != A->indptr[row + 1] && A->indices[lo] == col;
}

/* ILU0 (CG.h:257-284): factors on the pattern of A, row by row; q_ij -= q_ik q_kj
 * for k ascending while k < min(i, j); lower entries divided by q_jj.  The
 * factor keeps A's pattern, so q is stored directly in CSR (same get/set
 * results as the reference's LILCSR, which never adds entries here). */
int orc_ilu0(const orc_csr *A, orc_csr *M) {
    M->rows = A->rows;
    M->nnz = A->nnz;
    M->indptr = xmalloc(sizeof(int) * (A->rows + 1));
    M->indices = xmalloc(sizeof(int) * A->nnz);
    M->data = xmalloc(sizeof(double) * A->nnz);
    memcpy(M->indptr, A->indptr, sizeof(int) * (A->rows + 1));
    memcpy(M->indices, A->indices, sizeof(int) * A->nnz);
    memcpy(M->data, A->data, sizeof(double) * A->nnz);
    for (int i = 0; i < A->rows; i++) {
        for (int nidx = A->indptr[i]; nidx < A->indptr[i + 1]; nidx++) {
            int j = A->indices[nidx];
            double qij = A->data[nidx];
            /* the reference scans every k in [0, ROWS) and tests membership; only
               k in row i's pattern can pass, so walk row i's columns ascending */
            int lim = i <= j ? i : j;
            for (int kk = A->indptr[i]; kk < A->indptr[i + 1]; kk++) {
                int k = A->indices[kk];
                if (!csr_has(A, k, j)) continue;
                if (k < lim) qij -= orc_csr_get(M, i, k) * orc_csr_get(M, k, j);
                else break;
            }
            if (i > j) qij /= orc_csr_get(M, j, j);
            M->data[nidx] = qij;
        }
    }
    return 0;
}

/* PreILU0 (CG.h:288-315) */
void orc_pre_ilu0(const orc_csr *M, const double *b, double *v) {
    int n = M->rows;
    memcpy(v, b, sizeof(double) * n);
    for (int i = 0; i < n; i++)
        for (int k = M->indptr[i]; k < M->indptr[i + 1]; k++) {
            if (M->indices[k] < i) v[i] -= M->data[k] * v[M->indices[k]];
            else break;
        }
    for (int i = n - 1; i >= 0; i--) {
        for (int k = M->indptr[i + 1] - 1; k >= M->indptr[i]; k--) {
            if (M->indices[k] > i) v[i] -= M->data[k] * v[M->indices[k]];
            else break;
        }
        v[i] /= orc_csr_get(M, i, i);
    }
}

/* ILU0CG (CG.h:319-352) */
int orc_ilu0_cg(const orc_csr *A, const orc_csr *M, const double *b, int itmax, double eps,
                double *x) {
    long n = A->rows;
    size_t sz = sizeof(double) * n;
    double *r = xmalloc(sz), *p = xmalloc(sz), *Mr = xmalloc(sz), *Ap = xmalloc(sz);
    for (long i = 0; i < n; i++) x[i] = 0.0;
    orc_spmv(A, x, Ap);
    for (long i = 0; i < n; i++) r[i] = b[i] - Ap[i];
    orc_pre_ilu0(M, r, p);
    memcpy(Mr, p, sz);
    double bnorm = sqrt(dot(b, b, n));
    double Mrr = dot(Mr, r, n);
    int ret = -1;
    for (int k = 0; k < itmax; ++k) {
        orc_spmv(A, p, Ap);
        double alpha = Mrr / dot(p, Ap, n);
        for (long i = 0; i < n; i++) x[i] = x[i] + alpha * p[i];
        double ma = -alpha;
        for (long i = 0; i < n; i++) r[i] = r[i] + ma * Ap[i];
        orc_pre_ilu0(M, r, Mr);
        double Mrr1 = dot(Mr, r, n);
        double beta = Mrr1 / Mrr;
        for (long i = 0; i < n; i++) p[i] = beta * p[i] + Mr[i];
        Mrr = Mrr1;
        if (sqrt(dot(r, r, n)) < eps * bnorm) { ret = k + 1; break; }
    }
    free(r); free(p); free(Mr); free(Ap);
    return ret;
}

/* the preconditioned BiCGSTAB loop of ScalingBiCGSTAB (CG.h:457-495) and ILU0BiCGSTAB
 * (CG.h:356-391): M(v) is the preconditioner; p starts as M(r) for the scaling variant
 * (CG.h:463) and as r for the ILU(0) one (CG.h:362), as the reference writes them */
static int precond_bicgstab(const orc_csr *A, const double *b, int itmax, double eps, double *x,
                            void (*M)(const void *, const double *, double *), const void *ctx, int p_scaled) {
    long n = A->rows;
    size_t sz = sizeof(double) * n;
    double *r = xmalloc(sz), *rd = xmalloc(sz), *p = xmalloc(sz), *Mp = xmalloc(sz), *AMp = xmalloc(sz),
           *s = xmalloc(sz), *Ms = xmalloc(sz), *AMs = xmalloc(sz);
    for (long i = 0; i < n; i++) x[i] = 0.0;
    orc_spmv(A, x, AMp);
    for (long i = 0; i < n; i++) r[i] = b[i] - AMp[i];
    memcpy(rd, r, sz);
    if (p_scaled) M(ctx, r, p);
    else memcpy(p, r, sz);
    double rdr = dot(rd, r, n);
    double bnorm = sqrt(dot(b, b, n));
    int ret = -1;
    for (int k = 0; k < itmax; ++k) {
        M(ctx, p, Mp);
        orc_spmv(A, Mp, AMp);
        double alpha = rdr / dot(rd, AMp, n);
        double ma = -alpha;
        for (long i = 0; i < n; i++) s[i] = 1.0 * r[i] + ma * AMp[i];
        M(ctx, s, Ms);
        orc_spmv(A, Ms, AMs);
        double omega = dot(AMs, s, n) / dot(AMs, AMs, n);
        for (long i = 0; i < n; i++) x[i] = 1.0 * x[i] + alpha * Mp[i] + omega * Ms[i];
        double mo = -omega;
        for (long i = 0; i < n; i++) r[i] = 1.0 * s[i] + mo * AMs[i];
        double rdr1 = dot(rd, r, n);
        double beta = alpha / omega * rdr1 / rdr;
        double mbo = -beta * omega;
        for (long i = 0; i < n; i++) p[i] = beta * p[i] + 1.0 * r[i] + mbo * AMp[i];
        rdr = rdr1;
        if (sqrt(dot(r, r, n)) < eps * bnorm) { ret = k + 1; break; }
    }
    free(r); free(rd); free(p); free(Mp); free(AMp); free(s); free(Ms); free(AMs);
    return ret;
}

static void scaling_apply(const void *ctx, const double *v, double *out) {   /* Scaling :408-415 */
    const orc_csr *A = (const orc_csr *)ctx;
    for (int i = 0; i < A->rows; i++) out[i] = v[i] / orc_csr_get(A, i, i);
}
static void ilu0_apply(const void *ctx, const double *v, double *out) { orc_pre_ilu0((const orc_csr *)ctx, v, out); }

/* ScalingBiCGSTAB (CG.h:457-495) */
int orc_scaling_bicgstab(const orc_csr *A, const double *b, int itmax, double eps, double *x) {
    return precond_bicgstab(A, b, itmax, eps, x, scaling_apply, A, 1);
}

/* ILU0BiCGSTAB (CG.h:356-391) with the factor M of ILU0 */
int orc_ilu0_bicgstab(const orc_csr *A, const orc_csr *M, const double *b, int itmax, double eps, double *x) {
    return precond_bicgstab(A, b, itmax, eps, x, ilu0_apply, M, 0);
}

double orc_true_residual(const orc_csr *A, const double *b, const double *x) {
    long n = A->rows;
    double *Ax = xmalloc(sizeof(double) * n);
    orc_spmv(A, x, Ax);
    double rr = 0.0, bb = 0.0;
    for (long i = 0; i < n; i++) {
        double d = b[i] - Ax[i];
        rr += d * d;
        bb += b[i] * b[i];
    }
    free(Ax);
    return sqrt(rr) / sqrt(bb);
}

/* ===================== filters ===================== */
/* CenterOfGravity (General.h:70-77): sum of node coordinates, then / nen */
void orc_centroids(int ne, int nen, int dim, const int *conn, const double *coords, double *cg) {
    for (long e = 0; e < ne; e++) {
        double c[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < nen; i++)
            for (int k = 0; k < dim; k++) c[k] += coords[(long)conn[e * nen + i] * dim + k];
        for (int k = 0; k < dim; k++) cg[e * dim + k] = c[k] / (double)nen;
    }
}

/* (cg_i - cg_j).Norm() (Vector.h:223-230, 297-303) */
static inline double cg_dist(const double *a, const double *b, int dim) {
    double v = 0.0;
    for (int k = 0; k < dim; k++) v += pow(a[k] - b[k], 2.0);
    return sqrt(v);
}

long long orc_neighbors(int ne, int dim, const double *cg, double R, const int *grid, int *ptr,
                        int **idx_out, double **w_out) {
    long long cap = (long long)ne * 8 + 64, cnt = 0;
    int *idx = xmalloc(sizeof(int) * cap);
    double *w = xmalloc(sizeof(double) * cap);
    ptr[0] = 0;
    for (long i = 0; i < ne; i++) {
        const double *ci = cg + i * dim;
        if (!grid) {
            for (long j = 0; j < ne; j++) {
                double d = cg_dist(ci, cg + j * dim, dim);
                if (d <= R) {
                    if (cnt == cap) { cap *= 2; idx = realloc(idx, sizeof(int) * cap); w = realloc(w, sizeof(double) * cap); }
                    idx[cnt] = (int)j;
                    w[cnt] = (R - d) / R;
                    cnt++;
                }
            }
        } else {
            /* windowed search in ascending element id; the window is wider than R
               by more than one element, so it finds exactly the all-pairs list */
            int nx = grid[0], ny = grid[1], nz = grid[2];
            int ei, ej, ek = 0;
            if (nz > 0) { ek = (int)(i % nz); ej = (int)((i / nz) % ny); ei = (int)(i / ((long)nz * ny)); }
            else { ej = (int)(i % ny); ei = (int)(i / ny); }
            /* centroid spacing along each axis, from the first element's neighbours */
            long sx = nz > 0 ? (long)ny * nz : ny, sy = nz > 0 ? nz : 1;
            double hmin = 1e300;
            if (nx > 1) hmin = fmin(hmin, cg[sx * dim + 0] - cg[0]);
            if (ny > 1) hmin = fmin(hmin, cg[sy * dim + 1] - cg[1]);
            if (nz > 1) hmin = fmin(hmin, cg[1 * dim + 2] - cg[2]);
            if (!(hmin > 0.0) || hmin > 1e299) hmin = R > 0 ? R : 1.0;
            int W = (int)ceil(R / hmin) + 1;
            int i0 = ei - W < 0 ? 0 : ei - W, i1 = ei + W >= nx ? nx - 1 : ei + W;
            int j0 = ej - W < 0 ? 0 : ej - W, j1 = ej + W >= ny ? ny - 1 : ej + W;
            int k0 = 0, k1 = 0;
            if (nz > 0) { k0 = ek - W < 0 ? 0 : ek - W; k1 = ek + W >= nz ? nz - 1 : ek + W; }
            for (int a = i0; a <= i1; a++)
                for (int b = j0; b <= j1; b++)
                    for (int c = k0; c <= k1; c++) {
                        long j = nz > 0 ? ((long)ny * a + b) * nz + c : (long)ny * a + b;
                        double d = cg_dist(ci, cg + j * dim, dim);
                        if (d <= R) {
                            if (cnt == cap) { cap *= 2; idx = realloc(idx, sizeof(int) * cap); w = realloc(w, sizeof(double) * cap); }
                            idx[cnt] = (int)j;
                            w[cnt] = (R - d) / R;
                            cnt++;
                        }
                    }
        }
        ptr[i + 1] = (int)cnt;
    }
    *idx_out = idx;
    *w_out = w;
    return cnt;
}

/* DensityFilter::GetFilteredVariables (DensityFilter.h:44-56) */
void orc_density_filter(int n, const int *ptr, const int *idx, const double *w, const double *s,
                        double *rho) {
    for (int i = 0; i < n; i++) {
        double wsum = 0.0, r = 0.0;
        for (int k = ptr[i]; k < ptr[i + 1]; k++) {
            r += w[k] * s[idx[k]];
            wsum += w[k];
        }
        rho[i] = r / wsum;
    }
}

/* DensityFilter::GetFilteredSensitivitis (DensityFilter.h:59-71): divides by wsum_i */
void orc_density_filter_sens(int n, const int *ptr, const int *idx, const double *w,
                             const double *dfdrho, double *dfds) {
    for (int i = 0; i < n; i++) {
        double wsum = 0.0, v = 0.0;
        for (int k = ptr[i]; k < ptr[i + 1]; k++) {
            v += dfdrho[idx[k]] * w[k];
            wsum += w[k];
        }
        dfds[i] = v / wsum;
    }
}

/* SensitivityFilter::GetFilteredSensitivitis (Sigmund's scheme, SensitivityFilter.h:38-50),
 * mode 0: dfds_i = sum_j w_ij s_j d_j / (wsum_i s_i);
 * SensitivityFilter2 (Borrvall's scheme, :78-90), mode 1: / sum_j w_ij s_j */
void orc_sensitivity_filter(int n, const int *ptr, const int *idx, const double *w, const double *s,
                            const double *d, int mode, double *out) {
    for (int i = 0; i < n; i++) {
        double wsum = 0.0, v = 0.0;
        for (int k = ptr[i]; k < ptr[i + 1]; k++) {
            v += w[k] * s[idx[k]] * d[idx[k]];
            wsum += mode ? w[k] * s[idx[k]] : w[k];
        }
        out[i] = mode ? v / wsum : v / (wsum * s[i]);
    }
}

/* HeavisideFilter::GetFilteredVariables (HeavisideFilter.h:60-73) */
void orc_heaviside_filter(int n, const int *ptr, const int *idx, const double *w, double beta,
                          const double *s, double *rho) {
    for (int i = 0; i < n; i++) {
        double wssum = 0.0, wsum = 0.0;
        for (int k = ptr[i]; k < ptr[i + 1]; k++) {
            wssum += w[k] * s[idx[k]];
            wsum += w[k];
        }
        rho[i] = 0.5 * (tanh(0.5 * beta) + tanh(beta * (wssum / wsum - 0.5))) / tanh(0.5 * beta);
    }
}

/* HeavisideFilter::GetFilteredSensitivitis (HeavisideFilter.h:76-98) */
void orc_heaviside_filter_sens(int n, const int *ptr, const int *idx, const double *w, double beta,
                               const double *s, const double *dfdrho, double *dfds) {
    double *dr = xmalloc(sizeof(double) * n);
    for (int i = 0; i < n; i++) {
        double wssum = 0.0, wsum = 0.0;
        for (int k = ptr[i]; k < ptr[i + 1]; k++) {
            wssum += w[k] * s[idx[k]];
            wsum += w[k];
        }
        dr[i] = 0.5 * beta * (1.0 - pow(tanh(beta * (wssum / wsum - 0.5)), 2.0)) / tanh(0.5 * beta);
    }
    for (int i = 0; i < n; i++) {
        double wsum = 0.0, v = 0.0;
        for (int k = ptr[i]; k < ptr[i + 1]; k++) {
            v += dfdrho[idx[k]] * dr[idx[k]] * w[k];
            wsum += w[k];
        }
        dfds[i] = v / wsum;
    }
    free(dr);
}

/* ============ reaction, compliance, sensitivity (sample_optimize_density_oc.cpp:136-162) ============ */
double orc_compliance_sens(int kind, int nnodes, int ne, const int *conn, const double *coords,
                           const double *rho, double E1, double E0, double p, double V, double t,
                           double scale0, const double *u, double *r_out, double *dfdrho) {
    int nen, ndof, dim;
    orc_kind_shape(kind, &nen, &ndof, &dim);
    int nk = nen * ndof;
    long nd = (long)nnodes * ndof;
    double *RF = xcalloc(nd, sizeof(double));
    double *Ke = xmalloc(sizeof(double) * nk * nk), *ue = xmalloc(sizeof(double) * nk),
           *Ku = xmalloc(sizeof(double) * nk);
    double X[24];
    /* reaction: every dof numbered (RemoveBoundaryConditions + Renumbering), so n2g = node*ndof + d */
    for (int e = 0; e < ne; e++) {
        const int *en = conn + (long)e * nen;
        double E = E1 * pow(rho[e], p) + E0 * (1.0 - pow(rho[e], p));
        gather_X(nen, dim, en, coords, X);
        orc_ke(kind, X, E, V, t, Ke);
        for (int i = 0; i < nen; i++)
            for (int a = 0; a < ndof; a++) ue[ndof * i + a] = u[(long)en[i] * ndof + a];
        for (int i = 0; i < nk; i++) {                                  /* Matrix * Vector (Matrix.h:259-268) */
            double v = 0.0;
            for (int j = 0; j < nk; j++) v += Ke[i * nk + j] * ue[j];
            Ku[i] = v;
        }
        for (int i = 0; i < nen; i++)                                    /* Assembling(F, Fe) (Assembling.h:118-127) */
            for (int a = 0; a < ndof; a++) RF[(long)en[i] * ndof + a] += Ku[ndof * i + a];
    }
    /* f = scale0 * inner_product over nodes of u_node . r_node */
    double acc = 0.0;
    for (long nd_i = 0; nd_i < nnodes; nd_i++) {
        double v = 0.0;
        for (int a = 0; a < ndof; a++) v += u[nd_i * ndof + a] * RF[nd_i * ndof + a];
        acc = acc + v;
    }
    double f = scale0 * acc;
    /* sensitivities with the E = 1 element matrix */
    for (int e = 0; e < ne; e++) {
        const int *en = conn + (long)e * nen;
        gather_X(nen, dim, en, coords, X);
        orc_ke(kind, X, 1.0, V, t, Ke);
        for (int i = 0; i < nen; i++)
            for (int a = 0; a < ndof; a++) ue[ndof * i + a] = u[(long)en[i] * ndof + a];
        double q = 0.0;
        for (int i = 0; i < nk; i++) {
            double v = 0.0;
            for (int j = 0; j < nk; j++) v += Ke[i * nk + j] * ue[j];
            Ku[i] = v;
        }
        for (int i = 0; i < nk; i++) q += ue[i] * Ku[i];
        dfdrho[e] = -scale0 * p * (-E0 + E1) * pow(rho[e], p - 1.0) * q;
    }
    if (r_out) memcpy(r_out, RF, sizeof(double) * nd);
    free(RF); free(Ke); free(ue); free(Ku);
    return f;
}

/* ===================== OC (OC.h:67-107) ===================== */
int orc_is_convergence(double f, double prev, double eps) {
    return fabs(f - prev) / (f + prev) < eps;
}

static double volume_g(int n, const double *rho, double vf, double scale1) {
    double g = 0.0;                                   /* sample_optimize_density_oc.cpp:99-105 */
    for (int i = 0; i < n; i++) g += scale1 * rho[i] / (vf * n);
    return g - 1.0 * scale1;
}

double orc_oc_update(int n, double iota, double lmin, double lmax, double leps, double move,
                     double *xk, const double *dfdx, const double *dgdx, const int *ptr,
                     const int *idx, const double *w, double vf, double scale1, int heaviside,
                     double beta) {
    double l0 = lmin, l1 = lmax, lambda = 0.0;
    double *x1 = xcalloc(n, sizeof(double)), *rho = xmalloc(sizeof(double) * n);
    while ((l1 - l0) / (l1 + l0) > leps) {
        lambda = 0.5 * (l1 + l0);
        for (int i = 0; i < n; i++) {
            double v = pow(-dfdx[i] / (dgdx[i] * lambda), iota) * xk[i];
            double lo = smax(0.0, (1.0 - move) * xk[i]);
            double hi = smin(1.0, (1.0 + move) * xk[i]);
            if (v < lo) v = lo;
            else if (v > hi) v = hi;
            x1[i] = v;
        }
        /* the samples' constraint callback: re-filter and sum the volume */
        if (heaviside) orc_heaviside_filter(n, ptr, idx, w, beta, x1, rho);
        else orc_density_filter(n, ptr, idx, w, x1, rho);
        if (volume_g(n, rho, vf, scale1) > 0.0) l0 = lambda;
        else l1 = lambda;
    }
    memcpy(xk, x1, sizeof(double) * n);
    free(x1); free(rho);
    return lambda;
}

/* ===================== MMA (MMA.h) ===================== */
struct orc_mma {
    int k, n, m;
    double previousvalue, epsvalue;
    double *xmin, *xmax, *xkm2, *xkm1;
    double a0, *a, *c, *d;
    double raa0, albefa, move, asyinit, asydecr, asyincr;
    double *L, *U;
};

static double *dup(const double *s, int n) {
    double *p = xmalloc(sizeof(double) * (n > 0 ? n : 1));
    memcpy(p, s, sizeof(double) * n);
    return p;
}

/* MMA::MMA (MMA.h:63-88) */
orc_mma *orc_mma_create(int n, int m, double a0, const double *a, const double *c, const double *d,
                        const double *xmin, const double *xmax) {
    orc_mma *o = xcalloc(1, sizeof(orc_mma));
    o->k = 0; o->n = n; o->m = m;
    o->previousvalue = 0.0;
    o->epsvalue = 1.0e-5;
    o->xmin = dup(xmin, n); o->xmax = dup(xmax, n);
    o->xkm2 = xcalloc(n, sizeof(double)); o->xkm1 = xcalloc(n, sizeof(double));
    o->a0 = a0; o->a = dup(a, m); o->c = dup(c, m); o->d = dup(d, m);
    o->raa0 = 1.0e-5; o->albefa = 0.1; o->move = 0.5;
    o->asyinit = 0.5; o->asydecr = 0.7; o->asyincr = 1.2;
    o->L = xcalloc(n, sizeof(double)); o->U = xcalloc(n, sizeof(double));
    return o;
}

void orc_mma_set_parameters(orc_mma *o, double raa0, double albefa, double move, double asyinit,
                            double asydecr, double asyincr, double epsvalue) {
    o->raa0 = raa0; o->albefa = albefa; o->move = move; o->asyinit = asyinit;
    o->asydecr = asydecr; o->asyincr = asyincr; o->epsvalue = epsvalue;
}

int orc_mma_is_convergence(orc_mma *o, double f) {
    return fabs(f - o->previousvalue) / (f + o->previousvalue) < o->epsvalue;
}

void orc_mma_destroy(orc_mma *o) {
    if (!o) return;
    free(o->xmin); free(o->xmax); free(o->xkm2); free(o->xkm1); free(o->a); free(o->c);
    free(o->d); free(o->L); free(o->U); free(o);
}

/* MMA::solvels (MMA.h:464-509): Gauss elimination with partial pivoting, A is s x s */
static void mma_solvels(double *A, double *b, int s, double *x) {
    for (int i = 0; i < s - 1; i++) {
        double pivot = fabs(A[i * s + i]);
        int pi = i;
        for (int j = i + 1; j < s; j++)
            if (pivot < fabs(A[j * s + i])) { pivot = fabs(A[j * s + i]); pi = j; }
        if (pi != i) {
            double tmp = b[i]; b[i] = b[pi]; b[pi] = tmp;
            for (int j = i; j < s; j++) { tmp = A[i * s + j]; A[i * s + j] = A[pi * s + j]; A[pi * s + j] = tmp; }
        }
        for (int j = i + 1; j < s; j++) {
            for (int k = i + 1; k < s; k++) A[j * s + k] -= A[i * s + k] * A[j * s + i] / A[i * s + i];
            b[j] -= b[i] * A[j * s + i] / A[i * s + i];
        }
    }
    for (int i = s - 1; i >= 0; i--) {
        x[i] = b[i];
        for (int j = s - 1; j > i; j--) x[i] -= x[j] * A[i * s + j];
        x[i] /= A[i * s + i];
    }
}

/* MMA::KKTNorm (MMA.h:422-461) */
static double mma_kkt(const orc_mma *o, const double *x, const double *y, double z,
                      const double *lam, const double *gsi, const double *ita, const double *mu,
                      double zeta, const double *s, double eps, const double *p, const double *q,
                      const double *p0, const double *q0, const double *alpha, const double *beta,
                      const double *b, double *gbuf) {
    int n = o->n, m = o->m;
    double norm = 0.0;
    /* g_i accumulates over j in order (MMA.h:431-439); plambda/qlambda are
       per-j values, recomputed below where they are used */
    for (int i = 0; i < m; i++) gbuf[i] = 0.0;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++)
            gbuf[i] += p[(long)i * n + j] / (o->U[j] - x[j]) + q[(long)i * n + j] / (x[j] - o->L[j]);
    for (int j = 0; j < n; j++) {
        double plj = p0[j], qlj = q0[j];
        for (int i = 0; i < m; i++) {
            plj += lam[i] * p[(long)i * n + j];
            qlj += lam[i] * q[(long)i * n + j];
        }
        norm += pow(plj / pow(o->U[j] - x[j], 2.0) - qlj / pow(x[j] - o->L[j], 2.0) - gsi[j] + ita[j], 2.0);
        norm += pow(gsi[j] * (x[j] - alpha[j]) - eps, 2.0);
        norm += pow(ita[j] * (beta[j] - x[j]) - eps, 2.0);
    }
    for (int i = 0; i < m; i++) {
        norm += pow(o->c[i] + o->d[i] * y[i] - lam[i] - mu[i], 2.0);
        norm += pow(gbuf[i] - o->a[i] * z - y[i] + s[i] - b[i], 2.0);
        norm += pow(mu[i] * y[i] - eps, 2.0);
        norm += pow(lam[i] * s[i] - eps, 2.0);
    }
    double la = 0.0;
    for (int i = 0; i < m; i++) la = la + lam[i] * o->a[i];
    norm += pow(o->a0 - zeta - la, 2.0);
    norm += pow(zeta * z - eps, 2.0);
    return sqrt(norm);
}

static double max3(double a, double b, double c) { double r = a; if (r < b) r = b; if (r < c) r = c; return r; }
static double min3(double a, double b, double c) { double r = a; if (b < r) r = b; if (c < r) r = c; return r; }
static double max4(double a, double b, double c, double d) { double r = max3(a, b, c); if (r < d) r = d; return r; }
static double max5(double a, double b, double c, double d, double e) { double r = max4(a, b, c, d); if (r < e) r = e; return r; }

/* MMA::UpdateVariables (MMA.h:116-419) */
int orc_mma_update(orc_mma *o, double *xk, double f, const double *dfdx, const double *g,
                   const double *dgdx) {
    int n = o->n, m = o->m;
    double *L = o->L, *U = o->U, *xmin = o->xmin, *xmax = o->xmax;
    /* asymptotes (MMA.h:118-142) */
    if (o->k < 2) {
        for (int j = 0; j < n; j++) {
            L[j] = xk[j] - o->asyinit * (xmax[j] - xmin[j]);
            U[j] = xk[j] + o->asyinit * (xmax[j] - xmin[j]);
            L[j] = smin(smax(xk[j] - 10.0 * (xmax[j] - xmin[j]), L[j]), xk[j] - 0.01 * (xmax[j] - xmin[j]));
            U[j] = smin(smax(xk[j] + 0.01 * (xmax[j] - xmin[j]), U[j]), xk[j] + 10.0 * (xmax[j] - xmin[j]));
        }
    } else {
        for (int j = 0; j < n; j++) {
            double tmp = (xk[j] - o->xkm1[j]) * (o->xkm1[j] - o->xkm2[j]);
            if (tmp < 0.0) {
                L[j] = xk[j] - o->asydecr * (o->xkm1[j] - L[j]);
                U[j] = xk[j] + o->asydecr * (U[j] - o->xkm1[j]);
            } else if (tmp > 0.0) {
                L[j] = xk[j] - o->asyincr * (o->xkm1[j] - L[j]);
                U[j] = xk[j] + o->asyincr * (U[j] - o->xkm1[j]);
            } else {
                L[j] = xk[j] - (o->xkm1[j] - L[j]);
                U[j] = xk[j] + (U[j] - o->xkm1[j]);
            }
            L[j] = smin(smax(xk[j] - 10.0 * (xmax[j] - xmin[j]), L[j]), xk[j] - 0.01 * (xmax[j] - xmin[j]));
            U[j] = smin(smax(xk[j] + 0.01 * (xmax[j] - xmin[j]), U[j]), xk[j] + 10.0 * (xmax[j] - xmin[j]));
        }
    }
    size_t nb = sizeof(double) * (size_t)n, mb = sizeof(double) * (size_t)(m > 0 ? m : 1);
    double *alpha = xmalloc(nb), *beta = xmalloc(nb), *p0 = xmalloc(nb), *q0 = xmalloc(nb);
    double *p = xmalloc(nb * m), *q = xmalloc(nb * m), *b = xmalloc(mb);
    /* move limits (MMA.h:144-150) */
    for (int j = 0; j < n; j++) {
        alpha[j] = max3(xmin[j], L[j] + o->albefa * (xk[j] - L[j]), xk[j] - o->move * (xmax[j] - xmin[j]));
        beta[j] = min3(xmax[j], U[j] - o->albefa * (U[j] - xk[j]), xk[j] + o->move * (xmax[j] - xmin[j]));
    }
    /* p0, q0 (MMA.h:152-160) */
    for (int j = 0; j < n; j++) {
        double dp = smax(dfdx[j], 0.0), dm = smax(-dfdx[j], 0.0);
        p0[j] = pow(U[j] - xk[j], 2.0) * (1.001 * dp + 0.001 * dm + o->raa0 / (xmax[j] - xmin[j]));
        q0[j] = pow(xk[j] - L[j], 2.0) * (0.001 * dp + 1.001 * dm + o->raa0 / (xmax[j] - xmin[j]));
    }
    /* p, q, b (MMA.h:162-175) */
    for (int i = 0; i < m; i++) {
        b[i] = -g[i];
        for (int j = 0; j < n; j++) {
            double gij = dgdx[(long)i * n + j];
            double dp = smax(gij, 0.0), dm = smax(-gij, 0.0);
            p[(long)i * n + j] = pow(U[j] - xk[j], 2.0) * (1.001 * dp + 0.001 * dm + o->raa0 / (xmax[j] - xmin[j]));
            q[(long)i * n + j] = pow(xk[j] - L[j], 2.0) * (0.001 * dp + 1.001 * dm + o->raa0 / (xmax[j] - xmin[j]));
            b[i] += p[(long)i * n + j] / (U[j] - xk[j]) + q[(long)i * n + j] / (xk[j] - L[j]);
        }
    }
    /* interior point (MMA.h:177-411) */
    double eps = 1.0;
    double *x = xmalloc(nb), *gsi = xmalloc(nb), *ita = xmalloc(nb);
    double *y = xmalloc(mb), *lam = xmalloc(mb), *s = xmalloc(mb), *mu = xmalloc(mb);
    double z = 1.0, zeta = 1.0;
    for (int i = 0; i < m; i++) { y[i] = 1.0; lam[i] = 1.0; s[i] = 1.0; mu[i] = smax(1.0, 0.5 * o->c[i]); }
    for (int j = 0; j < n; j++) {
        x[j] = 0.5 * (alpha[j] + beta[j]);
        gsi[j] = smax(1.0, 1.0 / (x[j] - alpha[j]));
        ita[j] = smax(1.0, 1.0 / (beta[j] - x[j]));
    }
    double *G = xmalloc(nb * m), *Dx = xmalloc(nb), *dtx = xmalloc(nb), *dx = xmalloc(nb),
           *dgsi = xmalloc(nb), *dita = xmalloc(nb), *xp = xmalloc(nb), *gp = xmalloc(nb),
           *ip = xmalloc(nb);
    double *Dy = xmalloc(mb), *Dl = xmalloc(mb), *dty = xmalloc(mb), *dtl = xmalloc(mb),
           *Dly = xmalloc(mb), *dtly = xmalloc(mb), *dy = xmalloc(mb), *dl = xmalloc(mb),
           *dmu = xmalloc(mb), *ds = xmalloc(mb), *yp = xmalloc(mb), *lp = xmalloc(mb),
           *mp = xmalloc(mb), *sp = xmalloc(mb), *gb = xmalloc(mb);
    int S = (n > m ? m : n) + 1;
    double *A = xmalloc(sizeof(double) * S * S), *Bv = xmalloc(sizeof(double) * S),
           *sol = xmalloc(sizeof(double) * S);
    int newton = 0;
    for (int l = 0; eps > 1.0e-7; l++) {
        if (l >= 100000) break;   /* the reference has no cap; this only guards a runaway */
        newton++;
        /* coefficients */
        for (int i = 0; i < m; i++)
            for (int j = 0; j < n; j++)
                G[(long)i * n + j] = p[(long)i * n + j] / pow(U[j] - x[j], 2.0) - q[(long)i * n + j] / pow(x[j] - L[j], 2.0);
        for (int j = 0; j < n; j++) {
            double plj = p0[j], qlj = q0[j];
            for (int i = 0; i < m; i++) { plj += lam[i] * p[(long)i * n + j]; qlj += lam[i] * q[(long)i * n + j]; }
            Dx[j] = 2.0 * plj / pow(U[j] - x[j], 3.0) + 2.0 * qlj / pow(x[j] - L[j], 3.0) + gsi[j] / (x[j] - alpha[j]) + ita[j] / (beta[j] - x[j]);
            dtx[j] = plj / pow(U[j] - x[j], 2.0) - qlj / pow(x[j] - L[j], 2.0) - eps / (x[j] - alpha[j]) + eps / (beta[j] - x[j]);
        }
        for (int i = 0; i < m; i++) {
            Dy[i] = o->d[i] + mu[i] / y[i];
            Dl[i] = s[i] / lam[i];
            dty[i] = o->c[i] + o->d[i] * y[i] - lam[i] - eps / y[i];
        }
        double la = 0.0;
        for (int i = 0; i < m; i++) la = la + lam[i] * o->a[i];
        double dtz = o->a0 - eps / z - la;
        for (int i = 0; i < m; i++) {
            dtl[i] = -o->a[i] * z - y[i] - b[i] + eps / lam[i];
            for (int j = 0; j < n; j++) dtl[i] += p[(long)i * n + j] / (U[j] - x[j]) + q[(long)i * n + j] / (x[j] - L[j]);
            Dly[i] = Dl[i] + 1.0 / Dy[i];
            dtly[i] = dtl[i] + dty[i] / Dy[i];
        }
        double dz;
        /* Newton direction */
        if (n > m) {
            int s1 = m + 1;
            for (int k2 = 0; k2 < s1 * s1; k2++) A[k2] = 0.0;
            for (int ii = 0; ii < m; ii++) {
                for (int jj = 0; jj < m; jj++)
                    for (int kk = 0; kk < n; kk++)
                        A[ii * s1 + jj] += G[(long)ii * n + kk] * G[(long)jj * n + kk] / Dx[kk];
                A[ii * s1 + ii] += Dly[ii];
                A[ii * s1 + m] = o->a[ii];
                A[m * s1 + ii] = o->a[ii];
            }
            A[m * s1 + m] = -zeta / z;
            for (int ii = 0; ii < m; ii++) {
                Bv[ii] = dtly[ii];
                for (int jj = 0; jj < n; jj++) Bv[ii] -= G[(long)ii * n + jj] * dtx[jj] / Dx[jj];
            }
            Bv[m] = dtz;
            mma_solvels(A, Bv, s1, sol);
            for (int i = 0; i < m; i++) dl[i] = sol[i];
            dz = sol[m];
            for (int j = 0; j < n; j++) {
                dx[j] = -dtx[j] / Dx[j];
                for (int i = 0; i < m; i++) dx[j] -= G[(long)i * n + j] * dl[i] / Dx[j];
            }
        } else {
            int s1 = n + 1;
            for (int k2 = 0; k2 < s1 * s1; k2++) A[k2] = 0.0;
            for (int ii = 0; ii < n; ii++) {
                for (int jj = 0; jj < n; jj++)
                    for (int kk = 0; kk < m; kk++)
                        A[ii * s1 + jj] += G[(long)kk * n + ii] * G[(long)kk * n + jj] / Dly[kk];
                A[ii * s1 + ii] += Dx[ii];
                for (int jj = 0; jj < m; jj++) {
                    A[ii * s1 + n] -= G[(long)jj * n + ii] * o->a[jj] / Dly[jj];
                    A[n * s1 + ii] -= G[(long)jj * n + ii] * o->a[jj] / Dly[jj];
                    A[n * s1 + n] += o->a[jj] * o->a[jj] / Dly[jj];
                }
            }
            A[n * s1 + n] += zeta / z;
            for (int ii = 0; ii < n; ii++) {
                Bv[ii] = -dtx[ii];
                for (int jj = 0; jj < m; jj++) Bv[ii] -= G[(long)jj * n + ii] * dtly[jj] / Dly[jj];
            }
            Bv[n] = -dtz;
            for (int jj = 0; jj < m; jj++) Bv[n] += o->a[jj] * dtly[jj] / Dly[jj];
            mma_solvels(A, Bv, s1, sol);
            for (int j = 0; j < n; j++) dx[j] = sol[j];
            dz = sol[n];
            for (int i = 0; i < m; i++) {
                dl[i] = -o->a[i] * dz / Dly[i] + dtly[i] / Dly[i];
                for (int j = 0; j < n; j++) dl[i] += G[(long)i * n + j] * dx[j] / Dly[i];
            }
        }
        for (int i = 0; i < m; i++) {
            dy[i] = dl[i] / Dy[i] - dty[i] / Dy[i];
            dmu[i] = -mu[i] * dy[i] / y[i] - mu[i] + eps / y[i];
            ds[i] = -s[i] * dl[i] / lam[i] - s[i] + eps / lam[i];
        }
        for (int j = 0; j < n; j++) {
            dgsi[j] = -gsi[j] * dx[j] / (x[j] - alpha[j]) - gsi[j] + eps / (x[j] - alpha[j]);
            dita[j] = ita[j] * dx[j] / (beta[j] - x[j]) - ita[j] + eps / (beta[j] - x[j]);
        }
        double dzeta = -zeta * dz / z - zeta + eps / z;
        /* step length (MMA.h:345-360) */
        double txmax = 0.0;
        for (int j = 0; j < n; j++) {
            double t = max4(-1.01 * dx[j] / (x[j] - alpha[j]), 1.01 * dx[j] / (beta[j] - x[j]),
                            -1.01 * dgsi[j] / gsi[j], -1.01 * dita[j] / ita[j]);
            if (txmax < t) txmax = t;
        }
        double tymax = 0.0;
        for (int i = 0; i < m; i++) {
            double t = max4(-1.01 * dy[i] / y[i], -1.01 * dl[i] / lam[i], -1.01 * dmu[i] / mu[i],
                            -1.01 * ds[i] / s[i]);
            if (tymax < t) tymax = t;
        }
        double tau = 1.0 / max5(1.0, txmax, tymax, -1.01 * dz / z, -1.01 * dzeta / zeta);
        double dw = mma_kkt(o, x, y, z, lam, gsi, ita, mu, zeta, s, eps, p, q, p0, q0, alpha, beta, b, gb);
        double zp = z, zetap = zeta, dw1 = 0.0;
        /* backtracking (MMA.h:371-391) */
        for (int ll = 0; ll < 50; ll++) {
            for (int j = 0; j < n; j++) {
                xp[j] = x[j] + tau * dx[j];
                gp[j] = gsi[j] + tau * dgsi[j];
                ip[j] = ita[j] + tau * dita[j];
            }
            for (int i = 0; i < m; i++) {
                yp[i] = y[i] + tau * dy[i];
                lp[i] = lam[i] + tau * dl[i];
                mp[i] = mu[i] + tau * dmu[i];
                sp[i] = s[i] + tau * ds[i];
            }
            zp = z + tau * dz;
            zetap = zeta + tau * dzeta;
            dw1 = mma_kkt(o, xp, yp, zp, lp, gp, ip, mp, zetap, sp, eps, p, q, p0, q0, alpha, beta, b, gb);
            if (dw1 < dw) break;
            tau *= 0.5;
        }
        memcpy(x, xp, nb); memcpy(gsi, gp, nb); memcpy(ita, ip, nb);
        memcpy(y, yp, mb); memcpy(lam, lp, mb); memcpy(mu, mp, mb); memcpy(s, sp, mb);
        z = zp; zeta = zetap;
        double dw2 = mma_kkt(o, x, y, z, lam, gsi, ita, mu, zeta, s, eps, p, q, p0, q0, alpha, beta, b, gb);
        if (dw2 < 0.9 * eps) eps *= 0.1;
        else eps *= 1.0;
    }
    o->previousvalue = f;
    o->k++;
    memcpy(o->xkm2, o->xkm1, nb);
    memcpy(o->xkm1, xk, nb);
    memcpy(xk, x, nb);
    free(alpha); free(beta); free(p0); free(q0); free(p); free(q); free(b); free(x); free(gsi);
    free(ita); free(y); free(lam); free(s); free(mu); free(G); free(Dx); free(dtx); free(dx);
    free(dgsi); free(dita); free(xp); free(gp); free(ip); free(Dy); free(Dl); free(dty); free(dtl);
    free(Dly); free(dtly); free(dy); free(dl); free(dmu); free(ds); free(yp); free(lp); free(mp);
    free(sp); free(gb); free(A); free(Bv); free(sol);
    return newton;
}

/* ===================== CONLIN (src/Optimize/Solver/CONLIN.h) ===================== */
/* Convex linearisation: the same primal-dual interior-point subproblem solver as
 * MMA, on the approximation f~(x) = sum_j p_j x_j + q_j / x_j (terms linear in x_j
 * where the derivative is positive, in 1/x_j where it is negative) with plain move
 * limits and no asymptotes or history. */
struct orc_conlin {
    int k, n, m;
    double previousvalue, epsvalue, move;
    double *xmin, *xmax;
    double a0, *a, *c, *d;
};

/* CONLIN::CONLIN (CONLIN.h:55-67) */
orc_conlin *orc_conlin_create(int n, int m, double a0, const double *a, const double *c, const double *d,
                              const double *xmin, const double *xmax) {
    orc_conlin *o = xcalloc(1, sizeof(orc_conlin));
    o->k = 0; o->n = n; o->m = m;
    o->previousvalue = 0.0;
    o->epsvalue = 1.0e-5;
    o->move = 0.5;
    o->xmin = dup(xmin, n); o->xmax = dup(xmax, n);
    o->a0 = a0; o->a = dup(a, m); o->c = dup(c, m); o->d = dup(d, m);
    return o;
}

/* CONLIN::SetParameters (CONLIN.h:71-74) */
void orc_conlin_set_parameters(orc_conlin *o, double move, double epsvalue) {
    o->move = move;
    o->epsvalue = epsvalue;
}

/* CONLIN::IsConvergence (CONLIN.h:82-87) */
int orc_conlin_is_convergence(orc_conlin *o, double f) {
    return fabs(f - o->previousvalue) / (f + o->previousvalue) < o->epsvalue;
}

void orc_conlin_destroy(orc_conlin *o) {
    if (!o) return;
    free(o->xmin); free(o->xmax); free(o->a); free(o->c); free(o->d); free(o);
}

/* CONLIN::KKTNorm (CONLIN.h:369-407) */
static double conlin_kkt(const orc_conlin *o, const double *x, const double *y, double z,
                         const double *lam, const double *gsi, const double *ita, const double *mu,
                         double zeta, const double *s, double eps, const double *p, const double *q,
                         const double *p0, const double *q0, const double *alpha, const double *beta,
                         const double *b, double *gbuf) {
    int n = o->n, m = o->m;
    double norm = 0.0;
    for (int i = 0; i < m; i++) gbuf[i] = 0.0;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) gbuf[i] += p[(long)i * n + j] * x[j] + q[(long)i * n + j] / x[j];
    for (int j = 0; j < n; j++) {
        double plj = p0[j], qlj = q0[j];
        for (int i = 0; i < m; i++) {
            plj += lam[i] * p[(long)i * n + j];
            qlj += lam[i] * q[(long)i * n + j];
        }
        norm += pow(plj - qlj / pow(x[j], 2.0) - gsi[j] + ita[j], 2.0);
        norm += pow(gsi[j] * (x[j] - alpha[j]) - eps, 2.0);
        norm += pow(ita[j] * (beta[j] - x[j]) - eps, 2.0);
    }
    for (int i = 0; i < m; i++) {
        norm += pow(o->c[i] + o->d[i] * y[i] - lam[i] - mu[i], 2.0);
        norm += pow(gbuf[i] - o->a[i] * z - y[i] + s[i] - b[i], 2.0);
        norm += pow(mu[i] * y[i] - eps, 2.0);
        norm += pow(lam[i] * s[i] - eps, 2.0);
    }
    double la = 0.0;
    for (int i = 0; i < m; i++) la = la + lam[i] * o->a[i];
    norm += pow(o->a0 - zeta - la, 2.0);
    norm += pow(zeta * z - eps, 2.0);
    return sqrt(norm);
}

/* CONLIN::UpdateVariables (CONLIN.h:91-365).  Returns the interior-point Newton steps. */
int orc_conlin_update(orc_conlin *o, double *xk, double f, const double *dfdx, const double *g,
                      const double *dgdx) {
    int n = o->n, m = o->m;
    const double *xmin = o->xmin, *xmax = o->xmax;
    size_t nb = sizeof(double) * (size_t)n, mb = sizeof(double) * (size_t)(m > 0 ? m : 1);
    double *alpha = xmalloc(nb), *beta = xmalloc(nb), *p0 = xmalloc(nb), *q0 = xmalloc(nb);
    double *p = xmalloc(nb * m), *q = xmalloc(nb * m), *b = xmalloc(mb);
    /* move limits (CONLIN.h:92-97) */
    for (int j = 0; j < n; j++) {
        alpha[j] = smax(xmin[j], xk[j] - o->move * (xmax[j] - xmin[j]));
        beta[j] = smin(xmax[j], xk[j] + o->move * (xmax[j] - xmin[j]));
    }
    /* p0, q0 (CONLIN.h:100-107) */
    for (int j = 0; j < n; j++) {
        double dp = smax(dfdx[j], 0.0), dm = smax(-dfdx[j], 0.0);
        p0[j] = dp;
        q0[j] = dm * pow(xk[j], 2.0);
    }
    /* p, q, b (CONLIN.h:110-122) */
    for (int i = 0; i < m; i++) {
        b[i] = -g[i];
        for (int j = 0; j < n; j++) {
            double gij = dgdx[(long)i * n + j];
            double dp = smax(gij, 0.0), dm = smax(-gij, 0.0);
            p[(long)i * n + j] = dp;
            q[(long)i * n + j] = dm * pow(xk[j], 2.0);
            b[i] += p[(long)i * n + j] * xk[j] + q[(long)i * n + j] / xk[j];
        }
    }
    /* interior point (CONLIN.h:125-359) */
    double eps = 1.0;
    double *x = xmalloc(nb), *gsi = xmalloc(nb), *ita = xmalloc(nb);
    double *y = xmalloc(mb), *lam = xmalloc(mb), *s = xmalloc(mb), *mu = xmalloc(mb);
    double z = 1.0, zeta = 1.0;
    for (int i = 0; i < m; i++) { y[i] = 1.0; lam[i] = 1.0; s[i] = 1.0; mu[i] = smax(1.0, 0.5 * o->c[i]); }
    for (int j = 0; j < n; j++) {
        x[j] = 0.5 * (alpha[j] + beta[j]);
        gsi[j] = smax(1.0, 1.0 / (x[j] - alpha[j]));
        ita[j] = smax(1.0, 1.0 / (beta[j] - x[j]));
    }
    double *G = xmalloc(nb * m), *Dx = xmalloc(nb), *dtx = xmalloc(nb), *dx = xmalloc(nb),
           *dgsi = xmalloc(nb), *dita = xmalloc(nb), *xp = xmalloc(nb), *gp = xmalloc(nb),
           *ip = xmalloc(nb);
    double *Dy = xmalloc(mb), *Dl = xmalloc(mb), *dty = xmalloc(mb), *dtl = xmalloc(mb),
           *Dly = xmalloc(mb), *dtly = xmalloc(mb), *dy = xmalloc(mb), *dl = xmalloc(mb),
           *dmu = xmalloc(mb), *ds = xmalloc(mb), *yp = xmalloc(mb), *lp = xmalloc(mb),
           *mp = xmalloc(mb), *sp = xmalloc(mb), *gb = xmalloc(mb);
    int S = (n > m ? m : n) + 1;
    double *A = xmalloc(sizeof(double) * S * S), *Bv = xmalloc(sizeof(double) * S),
           *sol = xmalloc(sizeof(double) * S);
    int newton = 0;
    for (int l = 0; eps > 1.0e-7; l++) {
        if (l >= 100000) break;   /* the reference has no cap; this only guards a runaway */
        newton++;
        /* coefficients (CONLIN.h:148-195) */
        for (int i = 0; i < m; i++)
            for (int j = 0; j < n; j++)
                G[(long)i * n + j] = p[(long)i * n + j] - q[(long)i * n + j] / pow(x[j], 2.0);
        for (int j = 0; j < n; j++) {
            double plj = p0[j], qlj = q0[j];
            for (int i = 0; i < m; i++) { plj += lam[i] * p[(long)i * n + j]; qlj += lam[i] * q[(long)i * n + j]; }
            Dx[j] = 2.0 * qlj / pow(x[j], 3.0) + gsi[j] / (x[j] - alpha[j]) + ita[j] / (beta[j] - x[j]);
            dtx[j] = plj - qlj / pow(x[j], 2.0) - eps / (x[j] - alpha[j]) + eps / (beta[j] - x[j]);
        }
        for (int i = 0; i < m; i++) {
            Dy[i] = o->d[i] + mu[i] / y[i];
            Dl[i] = s[i] / lam[i];
            dty[i] = o->c[i] + o->d[i] * y[i] - lam[i] - eps / y[i];
        }
        double la = 0.0;
        for (int i = 0; i < m; i++) la = la + lam[i] * o->a[i];
        double dtz = o->a0 - eps / z - la;
        for (int i = 0; i < m; i++) {
            dtl[i] = -o->a[i] * z - y[i] - b[i] + eps / lam[i];
            for (int j = 0; j < n; j++) dtl[i] += p[(long)i * n + j] * x[j] + q[(long)i * n + j] / x[j];
            Dly[i] = Dl[i] + 1.0 / Dy[i];
            dtly[i] = dtl[i] + dty[i] / Dy[i];
        }
        double dz;
        /* Newton direction (CONLIN.h:197-291), both reductions */
        if (n > m) {
            int s1 = m + 1;
            for (int k2 = 0; k2 < s1 * s1; k2++) A[k2] = 0.0;
            for (int ii = 0; ii < m; ii++) {
                for (int jj = 0; jj < m; jj++)
                    for (int kk = 0; kk < n; kk++)
                        A[ii * s1 + jj] += G[(long)ii * n + kk] * G[(long)jj * n + kk] / Dx[kk];
                A[ii * s1 + ii] += Dly[ii];
                A[ii * s1 + m] = o->a[ii];
                A[m * s1 + ii] = o->a[ii];
            }
            A[m * s1 + m] = -zeta / z;
            for (int ii = 0; ii < m; ii++) {
                Bv[ii] = dtly[ii];
                for (int jj = 0; jj < n; jj++) Bv[ii] -= G[(long)ii * n + jj] * dtx[jj] / Dx[jj];
            }
            Bv[m] = dtz;
            mma_solvels(A, Bv, s1, sol);   /* CONLIN::solvels (CONLIN.h:411-455) is the same elimination */
            for (int i = 0; i < m; i++) dl[i] = sol[i];
            dz = sol[m];
            for (int j = 0; j < n; j++) {
                dx[j] = -dtx[j] / Dx[j];
                for (int i = 0; i < m; i++) dx[j] -= G[(long)i * n + j] * dl[i] / Dx[j];
            }
        } else {
            int s1 = n + 1;
            for (int k2 = 0; k2 < s1 * s1; k2++) A[k2] = 0.0;
            for (int ii = 0; ii < n; ii++) {
                for (int jj = 0; jj < n; jj++)
                    for (int kk = 0; kk < m; kk++)
                        A[ii * s1 + jj] += G[(long)kk * n + ii] * G[(long)kk * n + jj] / Dly[kk];
                A[ii * s1 + ii] += Dx[ii];
                for (int jj = 0; jj < m; jj++) {
                    A[ii * s1 + n] -= G[(long)jj * n + ii] * o->a[jj] / Dly[jj];
                    A[n * s1 + ii] -= G[(long)jj * n + ii] * o->a[jj] / Dly[jj];
                    A[n * s1 + n] += o->a[jj] * o->a[jj] / Dly[jj];
                }
            }
            A[n * s1 + n] += zeta / z;
            for (int ii = 0; ii < n; ii++) {
                Bv[ii] = -dtx[ii];
                for (int jj = 0; jj < m; jj++) Bv[ii] -= G[(long)jj * n + ii] * dtly[jj] / Dly[jj];
            }
            Bv[n] = -dtz;
            for (int jj = 0; jj < m; jj++) Bv[n] += o->a[jj] * dtly[jj] / Dly[jj];
            mma_solvels(A, Bv, s1, sol);
            for (int j = 0; j < n; j++) dx[j] = sol[j];
            dz = sol[n];
            for (int i = 0; i < m; i++) {
                dl[i] = -o->a[i] * dz / Dly[i] + dtly[i] / Dly[i];
                for (int j = 0; j < n; j++) dl[i] += G[(long)i * n + j] * dx[j] / Dly[i];
            }
        }
        for (int i = 0; i < m; i++) {
            dy[i] = dl[i] / Dy[i] - dty[i] / Dy[i];
            dmu[i] = -mu[i] * dy[i] / y[i] - mu[i] + eps / y[i];
            ds[i] = -s[i] * dl[i] / lam[i] - s[i] + eps / lam[i];
        }
        for (int j = 0; j < n; j++) {
            dgsi[j] = -gsi[j] * dx[j] / (x[j] - alpha[j]) - gsi[j] + eps / (x[j] - alpha[j]);
            dita[j] = ita[j] * dx[j] / (beta[j] - x[j]) - ita[j] + eps / (beta[j] - x[j]);
        }
        double dzeta = -zeta * dz / z - zeta + eps / z;
        /* step length (CONLIN.h:293-322) */
        double txmax = 0.0;
        for (int j = 0; j < n; j++) {
            double t = max4(-1.01 * dx[j] / (x[j] - alpha[j]), 1.01 * dx[j] / (beta[j] - x[j]),
                            -1.01 * dgsi[j] / gsi[j], -1.01 * dita[j] / ita[j]);
            if (txmax < t) txmax = t;
        }
        double tymax = 0.0;
        for (int i = 0; i < m; i++) {
            double t = max4(-1.01 * dy[i] / y[i], -1.01 * dl[i] / lam[i], -1.01 * dmu[i] / mu[i],
                            -1.01 * ds[i] / s[i]);
            if (tymax < t) tymax = t;
        }
        double tau = 1.0 / max5(1.0, txmax, tymax, -1.01 * dz / z, -1.01 * dzeta / zeta);
        double dw = conlin_kkt(o, x, y, z, lam, gsi, ita, mu, zeta, s, eps, p, q, p0, q0, alpha, beta, b, gb);
        double zp = z, zetap = zeta, dw1 = 0.0;
        /* backtracking on the KKT norm (CONLIN.h:323-339) */
        for (int ll = 0; ll < 50; ll++) {
            for (int j = 0; j < n; j++) {
                xp[j] = x[j] + tau * dx[j];
                gp[j] = gsi[j] + tau * dgsi[j];
                ip[j] = ita[j] + tau * dita[j];
            }
            for (int i = 0; i < m; i++) {
                yp[i] = y[i] + tau * dy[i];
                lp[i] = lam[i] + tau * dl[i];
                mp[i] = mu[i] + tau * dmu[i];
                sp[i] = s[i] + tau * ds[i];
            }
            zp = z + tau * dz;
            zetap = zeta + tau * dzeta;
            dw1 = conlin_kkt(o, xp, yp, zp, lp, gp, ip, mp, zetap, sp, eps, p, q, p0, q0, alpha, beta, b, gb);
            if (dw1 < dw) break;
            tau *= 0.5;
        }
        /* update w and eps (CONLIN.h:341-358) */
        memcpy(x, xp, nb); memcpy(gsi, gp, nb); memcpy(ita, ip, nb);
        memcpy(y, yp, mb); memcpy(lam, lp, mb); memcpy(mu, mp, mb); memcpy(s, sp, mb);
        z = zp; zeta = zetap;
        double dw2 = conlin_kkt(o, x, y, z, lam, gsi, ita, mu, zeta, s, eps, p, q, p0, q0, alpha, beta, b, gb);
        if (dw2 < 0.9 * eps) eps *= 0.1;
    }
    o->previousvalue = f;
    o->k++;
    memcpy(xk, x, nb);
    free(alpha); free(beta); free(p0); free(q0); free(p); free(q); free(b); free(x); free(gsi);
    free(ita); free(y); free(lam); free(s); free(mu); free(G); free(Dx); free(dtx); free(dx);
    free(dgsi); free(dita); free(xp); free(gp); free(ip); free(Dy); free(Dl); free(dty); free(dtl);
    free(Dly); free(dtly); free(dy); free(dl); free(dmu); free(ds); free(yp); free(lp); free(mp);
    free(sp); free(gb); free(A); free(Bv); free(sol);
    return newton;
}

/* ===================== the SIMP loop (sample_optimize_density_{oc,mma}.cpp) ===================== */
int orc_simp_run(const orc_simp_cfg *c, int iters, int stop_on_convergence, orc_simp_out *out) {
    int nen, ndof, dim;
    orc_kind_shape(c->kind, &nen, &ndof, &dim);
    int is3d = c->kind == ORC_H8_SOLID;
    long nnodes = is3d ? (long)(c->nx + 1) * (c->ny + 1) * (c->nz + 1) : (long)(c->nx + 1) * (c->ny + 1);
    int ne = is3d ? c->nx * c->ny * c->nz : c->nx * c->ny;
    double *coords = xmalloc(sizeof(double) * nnodes * dim);
    int *conn = xmalloc(sizeof(int) * (size_t)ne * nen);
    if (is3d) {
        orc_h8_nodes(c->lx, c->ly, c->lz, c->nx, c->ny, c->nz, coords);
        orc_h8_elements(c->nx, c->ny, c->nz, conn);
    } else {
        orc_q4_nodes(c->lx, c->ly, c->nx, c->ny, coords);
        orc_q4_elements(c->nx, c->ny, conn);
    }
    /* filter set-up (sample :43-63) */
    double *cg = xmalloc(sizeof(double) * ne * dim);
    orc_centroids(ne, nen, dim, conn, coords, cg);
    int *nptr = xmalloc(sizeof(int) * (ne + 1));
    int *nidx;
    double *nw;
    int grid[3] = {c->nx, c->ny, is3d ? c->nz : 0};
    orc_neighbors(ne, dim, cg, c->R, grid, nptr, &nidx, &nw);
    /* boundary conditions */
    unsigned char *fixed = xcalloc(nnodes * ndof, 1);
    for (int k = 0; k < c->nfix; k++) fixed[(long)c->fix_node[k] * ndof + c->fix_dof[k]] = 1;
    int *n2g = xmalloc(sizeof(int) * nnodes * ndof);

    double *s = xmalloc(sizeof(double) * ne), *rho = xmalloc(sizeof(double) * ne),
           *Ee = xmalloc(sizeof(double) * ne), *dfdrho = xmalloc(sizeof(double) * ne),
           *dgdrho = xmalloc(sizeof(double) * ne), *dfds = xmalloc(sizeof(double) * ne),
           *dgds = xmalloc(sizeof(double) * ne), *u = xmalloc(sizeof(double) * nnodes * ndof);
    for (int e = 0; e < ne; e++) s[e] = c->rho0;
    orc_mma *mma = NULL;
    orc_conlin *conlin = NULL;
    if (c->optimizer == 2) {
        /* sample_optimize_density_CONLIN.cpp:75-80: CONLIN(n, 1, a0, {0}, {c}, {d}, xmin, xmax),
           SetParameters(move, eps) */
        double *xmn = xmalloc(sizeof(double) * ne), *xmx = xmalloc(sizeof(double) * ne);
        for (int e = 0; e < ne; e++) { xmn[e] = c->mma_xmin; xmx[e] = c->mma_xmax; }
        double a = 0.0, cc = c->mma_c, dd = c->mma_d;
        conlin = orc_conlin_create(ne, 1, c->mma_a0, &a, &cc, &dd, xmn, xmx);
        orc_conlin_set_parameters(conlin, c->mma_move, c->mma_eps);
        free(xmn); free(xmx);
    }
    if (c->optimizer == 1) {
        double *xmn = xmalloc(sizeof(double) * ne), *xmx = xmalloc(sizeof(double) * ne);
        for (int e = 0; e < ne; e++) { xmn[e] = c->mma_xmin; xmx[e] = c->mma_xmax; }
        double a = 0.0, cc = c->mma_c, dd = c->mma_d;
        mma = orc_mma_create(ne, 1, c->mma_a0, &a, &cc, &dd, xmn, xmx);
        orc_mma_set_parameters(mma, c->mma_raa0, c->mma_albefa, c->mma_move, c->mma_asyinit,
                               c->mma_asydecr, c->mma_asyincr, c->mma_eps);
        free(xmn); free(xmx);
    }
    double oc_prev = 0.0, beta = 0.5;
    double ph[8] = {0};
    int done = 0;
    for (int k = 0; k < iters; k++) {
        double t0 = now_s();
        if (c->heaviside && k % 40 == 0) beta *= 2.0;
        if (c->heaviside) orc_heaviside_filter(ne, nptr, nidx, nw, beta, s, rho);
        else orc_density_filter(ne, nptr, nidx, nw, s, rho);
        double g = 0.0;
        for (int i = 0; i < ne; i++) {
            g += c->scale1 * rho[i] / (c->vf * ne);
            dgdrho[i] = c->scale1 / (c->vf * ne);
        }
        g -= 1.0 * c->scale1;
        double t1 = now_s();
        ph[0] += t1 - t0;
        /* displacement: SetDirichlet + Renumbering + assembly (sample :113-131) */
        for (long a = 0; a < nnodes * ndof; a++) u[a] = 0.0;
        int N = orc_renumber((int)nnodes, ndof, fixed, n2g);
        double *F = xcalloc(N, sizeof(double));
        for (int e = 0; e < ne; e++) Ee[e] = c->E1 * pow(rho[e], c->p) + c->E0 * (1.0 - pow(rho[e], c->p));
        orc_csr K;
        orc_assemble(c->kind, ne, conn, coords, Ee, c->V, c->t, n2g, NULL, N, &K, F);
        orc_neumann(c->nload, c->load_node, c->load_dof, c->load_val, ndof, n2g, F);
        double t2 = now_s();
        ph[1] += t2 - t1;
        double *res = xmalloc(sizeof(double) * N);
        int it = orc_scaling_cg(&K, F, c->cg_itmax, c->cg_eps, res);
        double t3 = now_s();
        ph[3] += t3 - t2;
        if (out && out->cg_iters) out->cg_iters[k] = it;
        if (out && out->true_res) out->true_res[k] = orc_true_residual(&K, F, res);
        for (long a = 0; a < nnodes * ndof; a++)                         /* Disassembling :162-171 */
            if (n2g[a] != -1) u[a] = res[n2g[a]];
        free(res); free(F);
        orc_csr_free(&K);
        double t4 = now_s();
        double f = orc_compliance_sens(c->kind, (int)nnodes, ne, conn, coords, rho, c->E1, c->E0, c->p,
                                       c->V, c->t, c->scale0, u, NULL, dfdrho);
        double t5 = now_s();
        ph[4] += t5 - t4;
        if (c->heaviside) {
            orc_heaviside_filter_sens(ne, nptr, nidx, nw, beta, s, dfdrho, dfds);
            orc_heaviside_filter_sens(ne, nptr, nidx, nw, beta, s, dgdrho, dgds);
        } else {
            orc_density_filter_sens(ne, nptr, nidx, nw, dfdrho, dfds);
            orc_density_filter_sens(ne, nptr, nidx, nw, dgdrho, dgds);
        }
        double t6 = now_s();
        ph[5] += t6 - t5;
        if (out) {
            if (out->f) out->f[k] = f;
            if (out->g) out->g[k] = g;
            if (out->rho) memcpy(out->rho + (long)k * ne, rho, sizeof(double) * ne);
            if (out->dfdrho) memcpy(out->dfdrho + (long)k * ne, dfdrho, sizeof(double) * ne);
            if (out->dfds) memcpy(out->dfds + (long)k * ne, dfds, sizeof(double) * ne);
            if (out->u) memcpy(out->u + (long)k * nnodes * ndof, u, sizeof(double) * nnodes * ndof);
        }
        int conv = c->optimizer == 1   ? orc_mma_is_convergence(mma, f)
                   : c->optimizer == 2 ? orc_conlin_is_convergence(conlin, f)
                                       : orc_is_convergence(f, oc_prev, 1.0e-5);
        if (stop_on_convergence && conv) { done = k + 1; break; }
        double lam = 0.0;
        int newton = 0;
        if (c->optimizer == 1) {
            newton = orc_mma_update(mma, s, f, dfds, &g, dgds);
        } else if (c->optimizer == 2) {
            newton = orc_conlin_update(conlin, s, f, dfds, &g, dgds);
        } else {
            lam = orc_oc_update(ne, c->oc_iota, c->oc_lmin, c->oc_lmax, c->oc_leps, c->oc_move, s,
                                dfds, dgds, nptr, nidx, nw, c->vf, c->scale1, c->heaviside, beta);
            oc_prev = f;
        }
        ph[6] += now_s() - t6;
        if (out) {
            if (out->lambda) out->lambda[k] = lam;
            if (out->mma_newton) out->mma_newton[k] = newton;
            if (out->s_after) memcpy(out->s_after + (long)k * ne, s, sizeof(double) * ne);
        }
        done = k + 1;
    }
    if (out && out->s_final) memcpy(out->s_final, s, sizeof(double) * ne);
    if (out && out->phase_seconds) memcpy(out->phase_seconds, ph, sizeof ph);
    orc_mma_destroy(mma);
    orc_conlin_destroy(conlin);
    free(coords); free(conn); free(cg); free(nptr); free(nidx); free(nw); free(fixed); free(n2g);
    free(s); free(rho); free(Ee); free(dfdrho); free(dgdrho); free(dfds); free(dgds); free(u);
    return done;
}
