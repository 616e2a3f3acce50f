/*
 * bem_oracle.c -- FP64 CPU restatement of the reference's Helmholtz BEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is built into
 * oracle/libbem_oracle.so and loaded by tests/, by __graft_entry__.smoke() and
 * by the cpu_baseline / --impl reference legs of bench.py.  The product library
 * (bem_gpu_clean_cpp_gb300) never links, loads or calls it.
 *
 * What it restates (file:line into the reference project
 * ZiqiFrancisFan/BEM_GPU_Clean_CPP):
 *   - Gauss-Legendre rule ............ numerical.cu:186-225 (GSL Golub-Welsch;
 *                                       here Newton on the Legendre recurrence)
 *   - Green's function, dG/dn ........ numerical.cu:70-74, mesh.cu:108-136
 *   - regular element integrals ...... mesh.cu:597-672 (g_h_c_l_nsgl)
 *   - vertex-singular integrals ...... mesh.cu:253-595, maps mesh.cu:1710-1729
 *   - system assembly + CHIEF rows ... atomicFuncs.cu:69-298, mesh.cu:985-1006
 *   - LS solve by Householder QR ..... numerical.cu:580-644 (cuSOLVER geqrf,
 *                                       unmqr, trsm in the reference)
 *   - unrestarted GMRES .............. GMRES.cu:26-279
 *   - field-point evaluation ......... mesh.cu:1008-1073
 *   - CHIEF candidate acceptance ..... mesh.cu:1119-1189,1411-1483,
 *                                       numerical.cu:105-131
 * plus one rule the reference lacks: adaptive subdivision for near-singular
 * pairs (dist(x, centroid) < eta * diam), used only when eta > 0.
 *
 * Parity pin: the oracle reproduces the reference's two committed golden
 * outputs (sphere171Hz_CHIEF, sphere171Hz_NoCHIEF; copies in tests/golden/)
 * from sphere.obj; see tests/test_oracle_golden.py.
 *
 * Complex numbers are C99 `double complex`; matrices are column-major with a
 * leading dimension, IDX(row,col,ld) = ld*col + row (numerical.h:44-46).
 */
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

#define ORC_PI 3.14159265358979323846
#define ORC_MAXQ 32
#define IDX(r, c, ld) ((size_t)(ld) * (size_t)(c) + (size_t)(r))

/* ------------------------------------------------------------------------ */
/* Parameters shared by the routines below (mirrors the reference's         */
/* __constant__ density/speed, numerical.cu:12-14, and INTORDER).           */
/* ------------------------------------------------------------------------ */
typedef struct {
    double density;   /* rho, 1.2041 in the reference                     */
    double speed;     /* c,   343.21 in the reference                     */
    int order;        /* Gauss points per direction, INTORDER = 6         */
    double near_eta;  /* 0: reference behaviour (plain rule for x not in e)*/
    int near_depth;   /* maximum subdivision depth for near-singular pairs */
} orc_params;

/* An incident field: kind 0 = point source q*G(k,|x-pos|) (pntSrc,
 * mesh.cu:114-118), kind 1 = plane wave a*exp(-i k d.x) (not in the reference;
 * e^{+i w t} convention like G). */
typedef struct {
    int kind;
    double vec[3];
    double amp_re, amp_im;
} orc_source;

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* Gauss-Legendre nodes/weights on [-1,1].  The reference builds the Jacobi */
/* matrix and calls gsl_eigen_symmv (numerical.cu:186-225); the nodes and   */
/* weights are the same numbers, produced here by Newton's method on the    */
/* three-term Legendre recurrence.  Nodes are returned in ascending order.  */
/* ------------------------------------------------------------------------ */
int orc_gauss_legendre(int n, double *x, double *w) {
    if (n < 1 || n > ORC_MAXQ) return 1;
    for (int i = 0; i < n; i++) {
        double z = cos(ORC_PI * (i + 0.75) / (n + 0.5));
        double dp = 0.0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int l = 2; l <= n; l++) {
                double p2 = ((2.0 * l - 1.0) * z * p1 - (l - 1.0) * p0) / l;
                p0 = p1;
                p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0; }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        /* recompute derivative at the converged node */
        double p0 = 1.0, p1 = z;
        for (int l = 2; l <= n; l++) {
            double p2 = ((2.0 * l - 1.0) * z * p1 - (l - 1.0) * p0) / l;
            p0 = p1;
            p1 = p2;
        }
        if (n == 1) { p1 = z; p0 = 1.0; }
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Geometry helpers                                                          */
/* ------------------------------------------------------------------------ */
static inline void sub3(const double *a, const double *b, double *o) {
    o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2];
}
static inline void cross3(const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
static inline double dot3(const double *a, const double *b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline double nrm3(const double *a) { return sqrt(dot3(a, a)); }

/* Green's function G = exp(-i k r)/(4 pi r)  (numerical.cu:70-74) */
static inline cplx green(double k, double r) {
    return (cos(k * r) - I * sin(k * r)) / (4.0 * ORC_PI * r);
}

/* Element geometry: normal n = (p1-p3)x(p2-p3) normalised, |J| = its norm
 * (mesh.cu:612-617). */
typedef struct {
    double p[3][3];
    double n[3];
    double J;
} orc_tri;

static void tri_setup(const double *p1, const double *p2, const double *p3, orc_tri *t) {
    double a[3], b[3], c[3];
    memcpy(t->p[0], p1, sizeof(double) * 3);
    memcpy(t->p[1], p2, sizeof(double) * 3);
    memcpy(t->p[2], p3, sizeof(double) * 3);
    sub3(p1, p3, a);
    sub3(p2, p3, b);
    cross3(a, b, c);
    t->J = nrm3(c);
    t->n[0] = c[0] / t->J; t->n[1] = c[1] / t->J; t->n[2] = c[2] / t->J;
}

/* Parent local coords -> physical point: xiToElem (mesh.cu:1692-1696). */
static inline void xi_to_elem(const orc_tri *t, double xi1, double xi2, double *y) {
    double xi3 = 1.0 - xi1 - xi2;
    for (int d = 0; d < 3; d++) y[d] = xi1 * t->p[0][d] + xi2 * t->p[1][d] + xi3 * t->p[2][d];
}

/*
 * Duffy (collapsed) tensor rule on a sub-triangle of the element.  The
 * sub-triangle has parent local vertices va, vb, vc (2-D); sub-local (s1,s2)
 * maps to xi = s1*va + s2*vb + (1-s1-s2)*vc.  `collapse` selects the map of the
 * unit square onto the triangle:
 *   3: s = (rho(1-theta), rho*theta)        -- regular rule and sgl3
 *                                             (mesh.cu:623-636, 1710-1714)
 *   1: s = (1-rho, rho(1-theta))            -- rhoThetaToXi_1 (mesh.cu:1716-1721)
 *   2: s = (rho*theta, 1-rho)               -- rhoThetaToXi_2 (mesh.cu:1723-1729)
 * with rho = (1+eta1)/2 (inner index m), theta = (1+eta2)/2 (outer index n),
 * weight 0.25*w_n*w_m*rho*|J|*|det(va-vc, vb-vc)|.
 * Accumulates  sg_j += w N_j G,  sh_j += w N_j dG/dn,  sc += w dG0/dn.
 */
static void rule_tri(double k, const double *x, const orc_tri *t,
                     const double *va, const double *vb, const double *vc, int collapse,
                     int nq, const double *gx, const double *gw,
                     cplx sg[3], cplx sh[3], double *sc) {
    double ea[2] = {va[0] - vc[0], va[1] - vc[1]};
    double eb[2] = {vb[0] - vc[0], vb[1] - vc[1]};
    double area_ratio = fabs(ea[0] * eb[1] - ea[1] * eb[0]);
    for (int n = 0; n < nq; n++) {
        double theta = 0.5 + 0.5 * gx[n];
        for (int m = 0; m < nq; m++) {
            double rho = 0.5 + 0.5 * gx[m];
            double s1, s2;
            if (collapse == 1) { s1 = 1.0 - rho; s2 = rho * (1.0 - theta); }
            else if (collapse == 2) { s1 = rho * theta; s2 = 1.0 - rho; }
            else { s1 = rho * (1.0 - theta); s2 = rho * theta; }
            double xi1 = vc[0] + s1 * ea[0] + s2 * eb[0];
            double xi2 = vc[1] + s1 * ea[1] + s2 * eb[1];
            double w = 0.25 * gw[n] * gw[m] * rho * t->J * area_ratio;
            double y[3], d[3];
            xi_to_elem(t, xi1, xi2, y);
            sub3(y, x, d);
            double r = nrm3(d);
            double drdn = dot3(d, t->n) / r;
            cplx G = green(k, r);
            cplx dG = G * (-1.0 / r - I * k) * drdn;       /* pGpn2, mesh.cu:130-136 */
            double dG0 = -drdn / (4.0 * ORC_PI * r * r);    /* pPsiLpn2, mesh.cu:125-128 */
            double N[3] = {xi1, xi2, 1.0 - xi1 - xi2};      /* N_1..3, mesh.cu:1656-1666 */
            for (int j = 0; j < 3; j++) {
                sg[j] += w * N[j] * G;
                sh[j] += w * N[j] * dG;
            }
            *sc += w * dG0;
        }
    }
}

static void near_rec(double k, const double *x, const orc_tri *t,
                     const double *va, const double *vb, const double *vc, int depth,
                     const orc_params *prm, const double *gx, const double *gw,
                     cplx sg[3], cplx sh[3], double *sc) {
    if (depth < prm->near_depth) {
        double yc[3], pa[3], pb[3], pc[3], d[3];
        double xc1 = (va[0] + vb[0] + vc[0]) / 3.0, xc2 = (va[1] + vb[1] + vc[1]) / 3.0;
        xi_to_elem(t, xc1, xc2, yc);
        xi_to_elem(t, va[0], va[1], pa);
        xi_to_elem(t, vb[0], vb[1], pb);
        xi_to_elem(t, vc[0], vc[1], pc);
        double dab[3], dbc[3], dca[3];
        sub3(pa, pb, dab); sub3(pb, pc, dbc); sub3(pc, pa, dca);
        double diam = fmax(nrm3(dab), fmax(nrm3(dbc), nrm3(dca)));
        sub3(yc, x, d);
        if (nrm3(d) < prm->near_eta * diam) {
            double mab[2] = {0.5 * (va[0] + vb[0]), 0.5 * (va[1] + vb[1])};
            double mbc[2] = {0.5 * (vb[0] + vc[0]), 0.5 * (vb[1] + vc[1])};
            double mca[2] = {0.5 * (vc[0] + va[0]), 0.5 * (vc[1] + va[1])};
            near_rec(k, x, t, va, mab, mca, depth + 1, prm, gx, gw, sg, sh, sc);
            near_rec(k, x, t, mab, vb, mbc, depth + 1, prm, gx, gw, sg, sh, sc);
            near_rec(k, x, t, mca, mbc, vc, depth + 1, prm, gx, gw, sg, sh, sc);
            near_rec(k, x, t, mab, mbc, mca, depth + 1, prm, gx, gw, sg, sh, sc);
            return;
        }
    }
    rule_tri(k, x, t, va, vb, vc, 3, prm->order, gx, gw, sg, sh, sc);
}

static const double V1[2] = {1.0, 0.0}, V2[2] = {0.0, 1.0}, V3[2] = {0.0, 0.0};

/*
 * g_j, h_j, c of one (point, element) pair.
 * sing = 0: x is not a vertex of the element -> regular rule (mesh.cu:597-672),
 *           or adaptive subdivision when eta > 0 and the pair is near.
 * sing = 1,2,3: x is vertex sing of the element -> vertex-collapsed rule
 *           (g/h/c_l_sgl1..3, mesh.cu:253-595).
 * g is multiplied by i*rho*omega, omega = k*speed (mesh.cu:667-669).
 * Returns 1 when the near-singular rule was used, else 0.
 */
int orc_elem_coeffs(double k, const double *x, const double *p1, const double *p2,
                    const double *p3, int sing, const orc_params *prm,
                    double *g_out /*6*/, double *h_out /*6*/, double *c_out) {
    double gx[ORC_MAXQ], gw[ORC_MAXQ];
    orc_gauss_legendre(prm->order, gx, gw);
    orc_tri t;
    tri_setup(p1, p2, p3, &t);
    cplx sg[3] = {0, 0, 0}, sh[3] = {0, 0, 0};
    double sc = 0.0;
    int used_near = 0;
    if (sing >= 1 && sing <= 3) {
        rule_tri(k, x, &t, V1, V2, V3, sing, prm->order, gx, gw, sg, sh, &sc);
    } else if (prm->near_eta > 0.0) {
        double yc[3], d[3], dab[3], dbc[3], dca[3];
        xi_to_elem(&t, 1.0 / 3.0, 1.0 / 3.0, yc);
        sub3(p1, p2, dab); sub3(p2, p3, dbc); sub3(p3, p1, dca);
        double diam = fmax(nrm3(dab), fmax(nrm3(dbc), nrm3(dca)));
        sub3(yc, x, d);
        if (nrm3(d) < prm->near_eta * diam) {
            used_near = 1;
            near_rec(k, x, &t, V1, V2, V3, 0, prm, gx, gw, sg, sh, &sc);
        } else {
            rule_tri(k, x, &t, V1, V2, V3, 3, prm->order, gx, gw, sg, sh, &sc);
        }
    } else {
        rule_tri(k, x, &t, V1, V2, V3, 3, prm->order, gx, gw, sg, sh, &sc);
    }
    double rw = prm->density * k * prm->speed;
    for (int j = 0; j < 3; j++) {
        cplx g = I * rw * sg[j];
        g_out[2 * j] = creal(g);
        g_out[2 * j + 1] = cimag(g);
        h_out[2 * j] = creal(sh[j]);
        h_out[2 * j + 1] = cimag(sh[j]);
    }
    *c_out = sc;
    return used_near;
}

/* Incident field at x: point source (pntSrc, mesh.cu:114-118) or plane wave. */
static cplx incident(double k, const orc_source *s, const double *x) {
    cplx a = s->amp_re + I * s->amp_im;
    if (s->kind == 1) {
        return a * cexp(-I * k * dot3(s->vec, x));
    }
    double d[3];
    sub3(x, s->vec, d);
    return a * green(k, nrm3(d));
}

/*
 * System assembly (bemSystem -> atomicGenSystem, mesh.cu:985-1006,
 * atomicFuncs.cu:218-298).  Rows 0..N-1 are the mesh nodes, rows N..N+M-1 the
 * CHIEF points (pts holds N+M points).  A is (N+M) x N, B is (N+M) x S.
 *   A = [I; 0], B[x,s] = p_inc_s(x)                  (atomicFuncs.cu:227-242)
 *   regular pairs (x not a vertex of e):             (atomicFuncs.cu:86-115)
 *     A[x,node_j] += h_j - (ca/cb) g_j;  A[x,x] -= c (x < N only);
 *     B[x,s] -= (cc/cb) sum_j g_j
 *   singular pairs (x = node_i of e), rule sgl_{i+1}: (atomicFuncs.cu:125-214)
 *     same three updates.
 * bc holds (ca, cb, cc) per element as 6 doubles (re, im); NULL means the
 * readObj default (0, 1, -1) (mesh.cu:1240-1242).
 * Only rows row_begin..row_end-1 are computed; A and B hold those rows
 * (local row x - row_begin).  Each row is independent; rows are spread over
 * OpenMP threads.
 */
int orc_assemble(int N, int M, const double *pts, int E, const int *elems, const double *bc,
                 double k, const orc_params *prm, int S, const orc_source *src,
                 double *A_ri, int lda, double *B_ri, int ldb, int row_begin, int row_end) {
    cplx *A = (cplx *)A_ri, *B = (cplx *)B_ri;
    int R = N + M;
    if (row_end < 0 || row_end > R) row_end = R;
    if (row_begin < 0) row_begin = 0;
    for (int e = 0; e < E; e++)
        for (int j = 0; j < 3; j++)
            if (elems[3 * e + j] < 0 || elems[3 * e + j] >= N) return 2;
    int err = 0;
#pragma omp parallel for schedule(dynamic, 4)
    for (int x = row_begin; x < row_end; x++) {
        const double *px = pts + 3 * (size_t)x;
        if (A) {
            for (int j = 0; j < N; j++) A[IDX(x - row_begin, j, lda)] = (x == j) ? 1.0 : 0.0;
        }
        cplx beta = 0.0;
        double csum = 0.0;
        for (int e = 0; e < E; e++) {
            const int *nd = elems + 3 * (size_t)e;
            cplx ca = 0.0, cb = 1.0, cc = -1.0;
            if (bc) {
                const double *b = bc + 6 * (size_t)e;
                ca = b[0] + I * b[1]; cb = b[2] + I * b[3]; cc = b[4] + I * b[5];
            }
            cplx bcA = ca / cb, bcC = cc / cb;
            int nsing = 0, which[3];
            if (x < N)
                for (int i = 0; i < 3; i++)
                    if (nd[i] == x) which[nsing++] = i + 1;
            int passes = nsing ? nsing : 1;
            for (int ps = 0; ps < passes; ps++) {
                double g[6], h[6], c;
                orc_elem_coeffs(k, px, pts + 3 * (size_t)nd[0], pts + 3 * (size_t)nd[1],
                                pts + 3 * (size_t)nd[2], nsing ? which[ps] : 0, prm, g, h, &c);
                cplx gs = 0.0;
                for (int j = 0; j < 3; j++) {
                    cplx gj = g[2 * j] + I * g[2 * j + 1];
                    cplx hj = h[2 * j] + I * h[2 * j + 1];
                    if (A) A[IDX(x - row_begin, nd[j], lda)] += hj - bcA * gj;
                    gs += gj;
                }
                if (x < N) csum += c;
                beta += bcC * gs;
            }
        }
        if (A && x < N) A[IDX(x - row_begin, x, lda)] -= csum;
        if (B) {
            for (int s = 0; s < S; s++) B[IDX(x - row_begin, s, ldb)] = incident(k, src + s, px) - beta;
        }
    }
    return err;
}

/*
 * Field evaluation (genExtPressure, mesh.cu:1008-1073), batched over points
 * and surface solutions:
 *   p(x) = p_inc(x) - sum_e [ sum_j (h_j - (ca/cb) g_j) p_j + (cc/cb) sum_j g_j ]
 * surfP is N x S (ldp), out is P x S (ldo).  Field points are never mesh
 * vertices, so only the regular (or near-singular) rule applies.
 */
int orc_field(int N, const double *pts, int E, const int *elems, const double *bc, double k,
              const orc_params *prm, int S, const orc_source *src, const double *surfP_ri,
              int ldp, int P, const double *fpts, double *out_ri, int ldo) {
    const cplx *surfP = (const cplx *)surfP_ri;
    cplx *out = (cplx *)out_ri;
#pragma omp parallel for schedule(dynamic, 1)
    for (int p = 0; p < P; p++) {
        const double *x = fpts + 3 * (size_t)p;
        cplx acc[64];
        int Sc = S < 64 ? S : 64;
        for (int s = 0; s < Sc; s++) acc[s] = 0.0;
        for (int e = 0; e < E; e++) {
            const int *nd = elems + 3 * (size_t)e;
            cplx ca = 0.0, cb = 1.0, cc = -1.0;
            if (bc) {
                const double *b = bc + 6 * (size_t)e;
                ca = b[0] + I * b[1]; cb = b[2] + I * b[3]; cc = b[4] + I * b[5];
            }
            cplx bcA = ca / cb, bcC = cc / cb;
            double g[6], h[6], c;
            orc_elem_coeffs(k, x, pts + 3 * (size_t)nd[0], pts + 3 * (size_t)nd[1],
                            pts + 3 * (size_t)nd[2], 0, prm, g, h, &c);
            cplx gs = 0.0, a[3];
            for (int j = 0; j < 3; j++) {
                cplx gj = g[2 * j] + I * g[2 * j + 1];
                a[j] = (h[2 * j] + I * h[2 * j + 1]) - bcA * gj;
                gs += gj;
            }
            for (int s = 0; s < Sc; s++) {
                cplx v = bcC * gs;
                for (int j = 0; j < 3; j++) v += a[j] * surfP[IDX(nd[j], s, ldp)];
                acc[s] += v;
            }
        }
        for (int s = 0; s < Sc; s++) out[IDX(p, s, ldo)] = incident(k, src + s, x) - acc[s];
    }
    return 0;
}

/*
 * Least-squares solve min ||A x - B|| by Householder QR, the algorithm
 * qrSolver (numerical.cu:580-644) delegates to cuSOLVER: A = QR (geqrf),
 * B := Q^H B (unmqr), R X = B(0:n) (trsm).  A (m x n, m >= n) is overwritten
 * by R and the reflectors; on return rows 0..n-1 of B hold X.
 */
int orc_lsq_qr(int m, int n, double *A_ri, int lda, double *B_ri, int nrhs, int ldb) {
    cplx *A = (cplx *)A_ri, *B = (cplx *)B_ri;
    if (m < n || n < 1) return 1;
    cplx *v = (cplx *)malloc(sizeof(cplx) * (size_t)m);
    for (int j = 0; j < n; j++) {
        int len = m - j;
        double xn2 = 0.0;
        for (int i = 0; i < len; i++) {
            cplx a = A[IDX(j + i, j, lda)];
            xn2 += creal(a) * creal(a) + cimag(a) * cimag(a);
        }
        double xn = sqrt(xn2);
        cplx x0 = A[IDX(j, j, lda)];
        double ax0 = cabs(x0);
        cplx ph = ax0 > 0 ? x0 / ax0 : 1.0;
        cplx alpha = -ph * xn;           /* new diagonal of R */
        for (int i = 0; i < len; i++) v[i] = A[IDX(j + i, j, lda)];
        v[0] -= alpha;
        double vn2 = 0.0;
        for (int i = 0; i < len; i++) vn2 += creal(v[i]) * creal(v[i]) + cimag(v[i]) * cimag(v[i]);
        if (vn2 == 0.0) continue;
        double tau = 2.0 / vn2;          /* H = I - tau v v^H */
        /* trailing columns of A */
#pragma omp parallel for schedule(static) if (n - j > 32)
        for (int c = j + 1; c < n; c++) {
            cplx s = 0.0;
            for (int i = 0; i < len; i++) s += conj(v[i]) * A[IDX(j + i, c, lda)];
            s *= tau;
            for (int i = 0; i < len; i++) A[IDX(j + i, c, lda)] -= s * v[i];
        }
        for (int c = 0; c < nrhs; c++) {
            cplx s = 0.0;
            for (int i = 0; i < len; i++) s += conj(v[i]) * B[IDX(j + i, c, ldb)];
            s *= tau;
            for (int i = 0; i < len; i++) B[IDX(j + i, c, ldb)] -= s * v[i];
        }
        A[IDX(j, j, lda)] = alpha;
        for (int i = 1; i < len; i++) A[IDX(j + i, j, lda)] = v[i];
    }
    free(v);
    /* back substitution R X = B(0:n) */
    for (int c = 0; c < nrhs; c++) {
        for (int i = n - 1; i >= 0; i--) {
            cplx s = B[IDX(i, c, ldb)];
            for (int l = i + 1; l < n; l++) s -= A[IDX(i, l, lda)] * B[IDX(l, c, ldb)];
            B[IDX(i, c, ldb)] = s / A[IDX(i, i, lda)];
        }
    }
    return 0;
}

/* y = A x (m x n, column-major) in FP64, OpenMP over rows. */
void orc_matvec(int m, int n, const double *A_ri, int lda, const double *x_ri, double *y_ri) {
    const cplx *A = (const cplx *)A_ri, *x = (const cplx *)x_ri;
    cplx *y = (cplx *)y_ri;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; i++) {
        cplx s = 0.0;
        for (int j = 0; j < n; j++) s += A[IDX(i, j, lda)] * x[j];
        y[i] = s;
    }
}

/*
 * Unrestarted GMRES on a square m x m system, restating GMRES.cu:145-279:
 * r = b - A x0; stop at once when ||r||/||b|| < thr; Arnoldi with modified
 * Gram-Schmidt (GMRES.cu:90-143), complex Givens rotations
 * (givens_coeffs/apply_givens, GMRES.cu:44-88), stop when
 * |err_i|/||b|| < thr or i >= maxIter, back-solve (Rsolver, GMRES.cu:26-42)
 * and x += Q y.  x holds x0 on entry and the solution on return.
 */
int orc_gmres(const double *A_ri, const double *b_ri, int m, int maxIter, double thr,
              double *x_ri, int *iters_out, double *relres_out) {
    const cplx *b = (const cplx *)b_ri;
    cplx *x = (cplx *)x_ri;
    int kmax = maxIter < m ? maxIter : m;
    if (kmax < 1) kmax = 1;
    cplx *Q = (cplx *)calloc((size_t)m * (kmax + 1), sizeof(cplx));
    cplx *H = (cplx *)calloc((size_t)(kmax + 1) * (kmax + 1), sizeof(cplx));
    cplx *cs = (cplx *)calloc(kmax + 1, sizeof(cplx));
    cplx *sn = (cplx *)calloc(kmax + 1, sizeof(cplx));
    cplx *err = (cplx *)calloc(kmax + 2, sizeof(cplx));
    cplx *r = (cplx *)malloc(sizeof(cplx) * m), *y = (cplx *)malloc(sizeof(cplx) * m);
    int ldh = kmax + 1;
    orc_matvec(m, m, A_ri, m, x_ri, (double *)r);
    double nb = 0.0, nr = 0.0;
    for (int i = 0; i < m; i++) {
        r[i] = b[i] - r[i];
        nb += creal(b[i]) * creal(b[i]) + cimag(b[i]) * cimag(b[i]);
        nr += creal(r[i]) * creal(r[i]) + cimag(r[i]) * cimag(r[i]);
    }
    nb = sqrt(nb); nr = sqrt(nr);
    int it = 0;
    if (nb == 0.0 || nr / nb < thr) {
        if (iters_out) *iters_out = 0;
        if (relres_out) *relres_out = nb > 0 ? nr / nb : 0.0;
        goto done;
    }
    err[0] = nr;
    for (int i = 0; i < m; i++) Q[i] = r[i] / nr;
    int i = 1;
    for (;;) {
        /* arnoldi step i: y = A q_{i-1}; MGS against q_0..q_{i-1} */
        orc_matvec(m, m, A_ri, m, (const double *)(Q + (size_t)(i - 1) * m), (double *)y);
        for (int l = 0; l < i; l++) {
            cplx h = 0.0;
            for (int t = 0; t < m; t++) h += conj(Q[(size_t)l * m + t]) * y[t];
            H[IDX(l, i - 1, ldh)] = h;
            for (int t = 0; t < m; t++) y[t] -= h * Q[(size_t)l * m + t];
        }
        double yn = 0.0;
        for (int t = 0; t < m; t++) yn += creal(y[t]) * creal(y[t]) + cimag(y[t]) * cimag(y[t]);
        yn = sqrt(yn);
        if (i < m) {
            H[IDX(i, i - 1, ldh)] = yn;
            if (i <= kmax && yn > 0)
                for (int t = 0; t < m; t++) Q[(size_t)i * m + t] = y[t] / yn;
        }
        /* apply previous rotations to column i-1, then the new one */
        cplx *h = H + (size_t)(i - 1) * ldh;
        for (int l = 0; l < i - 1; l++) {
            cplx t0 = cs[l] * h[l] + sn[l] * h[l + 1];
            cplx t1 = -conj(sn[l]) * h[l] + conj(cs[l]) * h[l + 1];
            h[l] = t0;
            h[l + 1] = t1;
        }
        if (i < m) {
            cplx rho = h[i - 1], sig = h[i];
            double mag = sqrt(cabs(rho) * cabs(rho) + cabs(sig) * cabs(sig));
            cs[i - 1] = conj(rho) / mag;
            sn[i - 1] = conj(sig) / mag;
            h[i - 1] = cs[i - 1] * h[i - 1] + sn[i - 1] * h[i];
            h[i] = 0.0;
            err[i] = -conj(sn[i - 1]) * err[i - 1];
            err[i - 1] = cs[i - 1] * err[i - 1];
        }
        if ((i < m && cabs(err[i]) / nb < thr) || i >= kmax) break;
        i++;
    }
    it = i;
    /* back substitution R y = err(0:it) */
    for (int l = it - 1; l >= 0; l--) {
        cplx s = err[l];
        for (int j = l + 1; j < it; j++) s -= H[IDX(l, j, ldh)] * y[j];
        y[l] = s / H[IDX(l, l, ldh)];
    }
    for (int t = 0; t < m; t++) {
        cplx s = 0.0;
        for (int l = 0; l < it; l++) s += Q[(size_t)l * m + t] * y[l];
        x[t] += s;
    }
    if (iters_out) *iters_out = it;
    if (relres_out) *relres_out = (it < m) ? cabs(err[it]) / nb : 0.0;
done:
    free(Q); free(H); free(cs); free(sn); free(err); free(r); free(y);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* CHIEF candidate acceptance (mesh::genCHIEF, mesh.cu:1430-1483).  The     */
/* candidates' uniform triples come from the caller (the reference draws    */
/* them with cuRAND's host XORWOW generator, one seed per candidate).       */
/* Candidate c: dir = (u0,u1,u2), point = lb + (ub-lb)*u (descale,          */
/* numerical.cu:105-107).  Accepted when the ray from the point along dir   */
/* crosses the surface an odd number of times (inObj, numerical.cu:119-131) */
/* and the point is at least `threshold` from every node (arrayMin,         */
/* numerical.cu:109-117).                                                   */
/* ------------------------------------------------------------------------ */
#define ORC_EPS 0.00005

static int ray_plane(const double *sp, const double *dir, const double *n, const double *p,
                     double *out) {
    /* rayPlaneInt, mesh.cu:1127-1146.  Returns 0 when the result is NaN. */
    double d[3];
    sub3(sp, p, d);
    if (dot3(n, d) == 0.0) { memcpy(out, sp, sizeof(double) * 3); return 1; }
    double nd = dot3(n, dir);
    if (nd == 0.0) return 0;
    double t = (dot3(n, p) - dot3(n, sp)) / nd;
    if (t > 0) {
        for (int i = 0; i < 3; i++) out[i] = sp[i] + t * dir[i];
        return 1;
    }
    return 0;
}

static int unit_or_nan(const double *v, double *o) {
    double nv = nrm3(v);
    if (nv == 0.0) return 0;
    o[0] = v[0] / nv; o[1] = v[1] / nv; o[2] = v[2] / nv;
    return 1;
}

static int close3(const double *a, const double *b) {
    return fabs(a[0] - b[0]) < ORC_EPS && fabs(a[1] - b[1]) < ORC_EPS && fabs(a[2] - b[2]) < ORC_EPS;
}

int orc_ray_tri(const double *sp, const double *dir, const double *p1, const double *p2,
                const double *p3) {
    /* rayTrnglInt (mesh.cu:1183-1189) + isInsideTrngl (mesh.cu:1164-1181) */
    double a[3], b[3], n[3], P[3];
    sub3(p2, p1, a);
    sub3(p3, p1, b);
    cross3(a, b, n);
    if (!ray_plane(sp, dir, n, p1, P)) return 0;
    double v12[3], v23[3], v31[3], v1p[3], v2p[3], v3p[3], t1[3], t2[3], t3[3], u1[3], u2[3], u3[3];
    sub3(p2, p1, v12); sub3(p3, p2, v23); sub3(p1, p3, v31);
    sub3(P, p1, v1p); sub3(P, p2, v2p); sub3(P, p3, v3p);
    cross3(v12, v1p, t1); cross3(v23, v2p, t2); cross3(v31, v3p, t3);
    if (!unit_or_nan(t1, u1) || !unit_or_nan(t2, u2) || !unit_or_nan(t3, u3)) return 0;
    return close3(u1, u2) && close3(u2, u3);
}

int orc_chief_select(int N, const double *pts, int E, const int *elems, const double *bb,
                     double threshold, int ncand, const double *cand, int num, double *out,
                     int *used) {
    int got = 0, c;
    for (c = 0; c < ncand && got < num; c++) {
        const double *u = cand + 3 * (size_t)c;
        double sp[3] = {bb[0] + (bb[1] - bb[0]) * u[0], bb[2] + (bb[3] - bb[2]) * u[1],
                        bb[4] + (bb[5] - bb[4]) * u[2]};
        int hits = 0;
        for (int e = 0; e < E; e++) {
            const int *nd = elems + 3 * (size_t)e;
            hits += orc_ray_tri(sp, u, pts + 3 * (size_t)nd[0], pts + 3 * (size_t)nd[1],
                                pts + 3 * (size_t)nd[2]);
        }
        double mind = 1e300;
        for (int i = 0; i < N; i++) {
            double d[3];
            sub3(pts + 3 * (size_t)i, sp, d);
            double r = nrm3(d);
            if (r < mind) mind = r;
        }
        if ((hits % 2 == 1) && !(mind < threshold)) {
            memcpy(out + 3 * (size_t)got, sp, sizeof(double) * 3);
            got++;
        }
    }
    if (used) *used = c;
    return got;
}
