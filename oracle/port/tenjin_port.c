/* CPU restatement ("port") of the Tenjin per-timestep update, FP64.
 * TEST INFRASTRUCTURE ONLY -- see tenjin_port.h. Citations are file:line in
 * the reference tree. Every expression keeps the reference's evaluation
 * order so that results agree bit for bit with the reference compiled on the
 * same machine; build with -ffp-contract=off.
 */
#include "tenjin_port.h"
#include "../shims/tj_libm.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Component map: AccessPattern (accesspattern.cpp:44-79).                  */
/* ------------------------------------------------------------------------ */
typedef struct {
    int ALPHA, ALPHARHO, RHO_K, RHO, RHOU, VEL, E, P, A, USTAR, SIGMA;
    int V, VSTAR, DEVH, HJ2, EPS, ARE;
    int RMIX, LAM, ARL; /* mixture: rhomix (2), lambda, alpharholambda; -1 without */
    int ncomp;
} cmap;

static cmap make_cmap(const tjp_params* p)
{
    cmap c;
    int n = 0, M = p->M;
    c.ALPHA = n; n += M;
    c.ALPHARHO = n; n += M;
    c.RHO_K = n; n += M;
    c.RHO = n; n += 1;
    c.RHOU = n; n += 3;
    c.VEL = n; n += 3;
    c.E = n; n += 1;
    c.P = n; n += 1;
    c.A = n; n += 1;
    c.USTAR = n; n += 1;
    c.SIGMA = n; n += 9;
    c.RMIX = c.LAM = c.ARL = -1;
    if (p->nmix) {
        c.RMIX = n; n += 2;
        c.LAM = n; n += 1;
        c.ARL = n; n += 1;
    }
    c.V = c.VSTAR = c.DEVH = c.HJ2 = c.EPS = c.ARE = -1;
    if (p->solid) {
        c.V = n; n += 9;
        c.VSTAR = n; n += 9;
        c.DEVH = n; n += 9;
        c.HJ2 = n; n += 1;
        if (p->plastic) {
            c.EPS = n; n += M;
            c.ARE = n; n += M;
        }
    }
    c.ncomp = n;
    return c;
}

int tjp_ncomp(const tjp_params* p) { return make_cmap(p).ncomp; }

int tjp_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Simulation state.                                                         */
/* ------------------------------------------------------------------------ */
typedef struct {
    int n[3];
    double dx[3];
    long N;
    int nbox;
    int* box;      /* 6 per box */
    int* cell_box; /* owning box of each valid cell */
    double *U1, *U, *U2, *UL, *UR;
    double* flux[3]; /* Ncomp per face, faces of direction d */
    long nf[3];
    /* THINC scratch: the alpha components of the reference's ULStar / URStar
     * CellArrays (hllc.cpp:622-623). ulstar/urstar hold the valid cells;
     * gstar[d] holds ULStar's ghost at each box's hi+1 face along d. */
    double *ulstar, *urstar, *gstar[3];
    double *candL, *candR;
    unsigned char *mixed, *flag, *tbv;
} pdom;

struct tjp_sim {
    tjp_params p;
    cmap c;
    int ndom;
    pdom* d;
    double dt;
    int err;
};

#define AT(arr, comp, cell) (arr)[(size_t)(comp) * (size_t)N + (size_t)(cell)]

static long lin(const pdom* D, int i, int j, int k) { return i + (long)D->n[0] * (j + (long)D->n[1] * k); }

/* Map a possibly-ghost index into the valid region; returns the sign for
 * components that are reflect_odd in a direction that reflected.
 * FillDomainBoundary semantics of the oracle shim (main.cpp:124-126). */
static void map_cell(const tjp_sim* s, const pdom* D, int* ijk, int* refl)
{
    for (int d = 0; d < 3; ++d) {
        refl[d] = 0;
        if (d >= s->p.dim) continue;
        int n = D->n[d];
        if (ijk[d] < 0) {
            if (s->p.lo_bc[d] == 1) { ijk[d] = -1 - ijk[d]; refl[d] = 1; }
            else ijk[d] = 0;
        } else if (ijk[d] > n - 1) {
            if (s->p.hi_bc[d] == 1) { ijk[d] = 2 * n - 1 - ijk[d]; refl[d] = 1; }
            else ijk[d] = n - 1;
        }
    }
}

static double odd_sign(const tjp_sim* s, int comp, const int* refl)
{
    double sg = 1.0;
    for (int d = 0; d < s->p.dim; ++d)
        if (refl[d] && (comp == s->c.VEL + d || comp == s->c.RHOU + d)) sg = -sg;
    return sg;
}

/* Value of component comp of array arr at (possibly ghost) cell i,j,k. */
static double gv(const tjp_sim* s, const pdom* D, const double* arr, int comp, int i, int j, int k)
{
    int ijk[3] = {i, j, k}, refl[3];
    map_cell(s, D, ijk, refl);
    long N = D->N;
    double v = AT(arr, comp, lin(D, ijk[0], ijk[1], ijk[2]));
    return odd_sign(s, comp, refl) < 0.0 ? -v : v;
}

/* ------------------------------------------------------------------------ */
/* Small-tensor algebra (tensor.cpp).                                       */
/* ------------------------------------------------------------------------ */
static double det2(double a, double b, double c, double d) { return a * d - b * c; }

/* det: recursive cofactor expansion along the first row (tensor.cpp:296-333) */
static double det3(const double* M)
{
    double det = 0.0;
    det += (1.0 * M[0]) * det2(M[4], M[5], M[7], M[8]);
    det += (-1.0 * M[1]) * det2(M[3], M[5], M[6], M[8]);
    det += (1.0 * M[2]) * det2(M[3], M[4], M[6], M[7]);
    return det;
}

/* invert: cofactor transpose over det (tensor.cpp:187-233) */
static void invert3(const double* M, double* Minv)
{
    double D = det3(M), cof[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double sub[4];
            int c = 0;
            for (int k = 0; k < 3; ++k)
                for (int m = 0; m < 3; ++m)
                    if (!(k == i || m == j)) sub[c++] = M[k * 3 + m];
            double sg = ((i + j) % 2) ? -1.0 : 1.0;
            cof[i * 3 + j] = sg * det2(sub[0], sub[1], sub[2], sub[3]);
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Minv[i * 3 + j] = cof[j * 3 + i] / D;
}

/* dgemm, row-major, k summed innermost in increasing order (tensor.cpp:81-115) */
static void mm(const double* A, const double* B, double* C)
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int l = 0; l < 3; ++l) s += A[i * 3 + l] * B[l * 3 + j];
            C[i * 3 + j] = s;
        }
}
static void mmT(const double* A, const double* B, double* C) /* A B^T */
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int l = 0; l < 3; ++l) s += A[i * 3 + l] * B[j * 3 + l];
            C[i * 3 + j] = s;
        }
}
static double trace3(const double* M) { double t = 0.0; t += M[0]; t += M[4]; t += M[8]; return t; }

/* Symmetric 3x3 eigendecomposition by cyclic Jacobi rotations (Golub & Van
 * Loan sec. 8.5): the stand-in for LAPACK dgesdd on symmetric positive
 * definite input. w decreasing, q eigenvectors as columns. */
static void sym3_eig(const double* a_in, double* w, double* q)
{
    double a[9];
    for (int i = 0; i < 9; ++i) a[i] = a_in[i];
    for (int i = 0; i < 9; ++i) q[i] = (i % 4 == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = fabs(a[1]) + fabs(a[2]) + fabs(a[5]);
        if (off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int r = p + 1; r < 3; ++r) {
                double apr = a[p * 3 + r];
                if (apr == 0.0) continue;
                double app = a[p * 3 + p], arr = a[r * 3 + r];
                double theta = (arr - app) / (2.0 * apr);
                double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0);
                double s = t * c;
                for (int k = 0; k < 3; ++k) {
                    double akp = a[k * 3 + p], akr = a[k * 3 + r];
                    a[k * 3 + p] = c * akp - s * akr;
                    a[k * 3 + r] = s * akp + c * akr;
                }
                for (int k = 0; k < 3; ++k) {
                    double apk = a[p * 3 + k], ark = a[r * 3 + k];
                    a[p * 3 + k] = c * apk - s * ark;
                    a[r * 3 + k] = s * apk + c * ark;
                }
                a[p * 3 + r] = 0.0;
                a[r * 3 + p] = 0.0;
                for (int k = 0; k < 3; ++k) {
                    double qkp = q[k * 3 + p], qkr = q[k * 3 + r];
                    q[k * 3 + p] = c * qkp - s * qkr;
                    q[k * 3 + r] = s * qkp + c * qkr;
                }
            }
    }
    int order[3] = {0, 1, 2};
    double d[3] = {a[0], a[4], a[8]};
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (d[order[j]] > d[order[i]]) { int t = order[i]; order[i] = order[j]; order[j] = t; }
    double qs[9];
    for (int c = 0; c < 3; ++c) {
        w[c] = d[order[c]];
        for (int r = 0; r < 3; ++r) qs[r * 3 + c] = q[r * 3 + order[c]];
    }
    for (int i = 0; i < 9; ++i) q[i] = qs[i];
}

/* matrixSquareRoot (tensor.cpp:452-475): L S^(1/2) RT with L = Q, RT = Q^T,
 * both products through dgemm. */
static void sqrtm3(const double* A, double* R)
{
    double w[3], q[9], L[9], RT[9], S[9], tmp[9];
    sym3_eig(A, w, q);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            L[i * 3 + j] = q[i * 3 + j];
            RT[i * 3 + j] = q[j * 3 + i];
            S[i * 3 + j] = sqrt(w[i]) * (double)(i == j);
        }
    mm(L, S, tmp);
    mm(tmp, RT, R);
}

/* ------------------------------------------------------------------------ */
/* Equations of state (equationofstate.cpp; copper class in ref_harness).   */
/* A cell view: the values the EOS reads.                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
    double alpha, arho, rhok, p, hj2;
    double lam, rm0, rm1; /* MixtureEOS only: lambda, rhomix rows 0 and 1 */
} ecell;

static double Gam(const tjp_sim* s, int m) { return s->p.eos_params[m][0] - 1.0; }
#define PRM(m, q) (s->p.eos_params[m][q])

/* MixtureEOS (equationofstate.cpp:117-396): two stiffened gases
 * [gamma, pref, eref, CV] x 2 blended by lambda; GruneisenGamma = gamma - 1. */
#define MG1(m) (PRM(m, 0) - 1.0)
#define MG2(m) (PRM(m, 4) - 1.0)
static double mix_gamma_term(const tjp_sim* s, int m, double lam) /* :175, :224 */
{
    return (lam * PRM(m, 0) * PRM(m, 3) + (1.0 - lam) * PRM(m, 4) * PRM(m, 7)) / (lam * PRM(m, 3) + (1.0 - lam) * PRM(m, 7)) -
           1.0;
}

static double eos_e_cold(const tjp_sim* s, int m, const ecell* e)
{
    double x;
    switch (s->p.eos[m]) {
        case 0: return PRM(m, 2) * e->arho; /* equationofstate.cpp:37-40 */
        case 4: /* :161-165 */
            return e->lam * (PRM(m, 2) * e->arho) + (1.0 - e->lam) * (PRM(m, 6) * e->arho);
        case 1: {
            double a = PRM(m, 6), K0 = PRM(m, 5), r0 = PRM(m, 4);
            x = e->rhok / r0;
            return e->arho * (((K0 / (2.0 * r0 * a * a)) * (tjm_pow(x, a) - 1.0)) * (tjm_pow(x, a) - 1.0));
        }
        case 2: {
            double r0 = PRM(m, 4);
            x = e->rhok / r0;
            return e->arho * ((PRM(m, 5) + PRM(m, 6) * x * x + PRM(m, 7) * x + PRM(m, 8) / x - PRM(m, 9) * tjm_log(x)) / r0);
        }
        default: {
            double r0 = PRM(m, 4), c0 = PRM(m, 5), sl = PRM(m, 6);
            double et = 1.0 - r0 / e->rhok, dd = 1.0 - sl * et;
            double ph = r0 * c0 * c0 * et / (dd * dd);
            return e->arho * (ph * et / (2.0 * r0));
        }
    }
}

static double eos_p_cold(const tjp_sim* s, int m, const ecell* e)
{
    double G = Gam(s, m), x;
    switch (s->p.eos[m]) {
        case 0: return PRM(m, 1) * e->alpha / G; /* equationofstate.cpp:42-45 */
        case 4: /* :167-171 */
            return (PRM(m, 1) * e->alpha / MG1(m)) * e->lam * e->rhok / (e->rm0) +
                   (PRM(m, 5) * e->alpha / MG2(m)) * (1.0 - e->lam) * e->rhok / (e->rm1);
        case 1: {
            double a = PRM(m, 6), K0 = PRM(m, 5), r0 = PRM(m, 4);
            x = e->rhok / r0;
            return (e->alpha / G) * ((K0 / a) * tjm_pow(x, a + 1.0) * (tjm_pow(x, a) - 1.0));
        }
        case 2: {
            double r0 = PRM(m, 4);
            x = e->rhok / r0;
            return (e->alpha / G) * ((2.0 * PRM(m, 6) * x * x * x + PRM(m, 7) * x * x - PRM(m, 8) - PRM(m, 9) * x));
        }
        default: {
            double r0 = PRM(m, 4), c0 = PRM(m, 5), sl = PRM(m, 6);
            double et = 1.0 - r0 / e->rhok, dd = 1.0 - sl * et;
            double ph = r0 * c0 * c0 * et / (dd * dd);
            return (e->alpha / G) * ph;
        }
    }
}

static double eos_G(const tjp_sim* s, int m, const ecell* e)
{
    switch (s->p.eos[m]) {
        case 0: return 0.0 * e->alpha;
        case 4: return 0.0;
        case 1: return PRM(m, 8) * tjm_pow((e->rhok / PRM(m, 4)), PRM(m, 7) + 1.0);
        case 2: return PRM(m, 10);
        default: return PRM(m, 7);
    }
}

static double eos_dGdrho(const tjp_sim* s, int m, const ecell* e)
{
    switch (s->p.eos[m]) {
        case 0: return 0.0 * e->alpha;
        case 1: {
            double b = PRM(m, 7), r0 = PRM(m, 4);
            return PRM(m, 8) * (b + 1.0) * tjm_pow((e->rhok / r0), b) / r0;
        }
        default: return 0.0;
    }
}

static double eos_dG2drho2(const tjp_sim* s, int m, const ecell* e)
{
    switch (s->p.eos[m]) {
        case 0: return 0.0 * e->alpha;
        case 1: {
            double b = PRM(m, 7), r0 = PRM(m, 4);
            return PRM(m, 8) * (b + 1.0) * (b)*tjm_pow((e->rhok / r0), b - 1.0) / (r0 * r0);
        }
        default: return 0.0;
    }
}

static double eos_e_shear(const tjp_sim* s, int m, const ecell* e)
{
    switch (s->p.eos[m]) {
        case 0: return 0.0 * e->alpha;
        case 4: return 0.0;
        case 3: return e->alpha * (PRM(m, 7) * e->hj2);
        default: return e->alpha * (eos_G(s, m, e) * e->hj2);
    }
}

static double eos_p_shear(const tjp_sim* s, int m, const ecell* e)
{
    double G = Gam(s, m);
    switch (s->p.eos[m]) {
        case 0: return 0.0 * e->alpha;
        case 4: return 0.0;
        case 3: return (e->alpha / G) * ((e->rhok * 0.0 - PRM(m, 7)) * e->hj2);
        default: return (e->alpha / G) * ((e->rhok * eos_dGdrho(s, m, e) - eos_G(s, m, e)) * e->hj2);
    }
}

static double eos_invG(const tjp_sim* s, int m, const ecell* e)
{
    if (s->p.eos[m] == 4) return e->alpha / mix_gamma_term(s, m, e->lam); /* :173-178 */
    return e->alpha / Gam(s, m);
}

/* xi (equationofstate.cpp:72-75, 222-225) */
static double eos_xi(const tjp_sim* s, int m, const ecell* e)
{
    if (s->p.eos[m] == 4) return 1.0 / mix_gamma_term(s, m, e->lam);
    return 1.0 / Gam(s, m);
}

static double eos_c2(const tjp_sim* s, int m, const ecell* e)
{
    double G = Gam(s, m);
    switch (s->p.eos[m]) {
        case 0: return e->p * (G + 1.0) / e->rhok - PRM(m, 1) / e->rhok; /* :61-64 */
        case 4: { /* mixtureSoundSpeed (:208-220) */
            double dedrho = (e->lam) * ((PRM(m, 1) - e->p) / (MG1(m) * e->rhok * e->rhok));
            dedrho += (1.0 - e->lam) * ((PRM(m, 5) - e->p) / (MG2(m) * e->rhok * e->rhok));
            return (e->p / (e->rhok * e->rhok) - dedrho) /
                   (e->lam / (e->rm0 * MG1(m)) + (1.0 - e->lam) / (e->rm1 * MG2(m)));
        }
        case 1: {
            double a = PRM(m, 6), K0 = PRM(m, 5), r0 = PRM(m, 4), x = e->rhok / r0;
            double dpc = (K0 / (a * r0)) * tjm_pow(x, a) * ((2.0 * a + 1.0) * tjm_pow(x, a) - (a + 1.0));
            double dps = e->rhok * eos_dG2drho2(s, m, e) * e->hj2;
            return (e->p * (G + 1.0) - (eos_p_cold(s, m, e) + eos_p_shear(s, m, e)) * (G + 1.0)) / e->rhok + dpc + dps +
                   (4.0 / 3.0) * eos_G(s, m, e) / e->rhok;
        }
        case 2: {
            double r0 = PRM(m, 4), x = e->rhok / r0;
            double dpc = (6.0 * PRM(m, 6) * x * x + 2.0 * PRM(m, 7) * x - PRM(m, 9)) / r0;
            double dps = e->rhok * eos_dG2drho2(s, m, e) * e->hj2;
            return (e->p * (G + 1.0) - (eos_p_cold(s, m, e) + eos_p_shear(s, m, e)) * (G + 1.0)) / e->rhok + dpc + dps +
                   (4.0 / 3.0) * eos_G(s, m, e) / e->rhok;
        }
        default: {
            double r0 = PRM(m, 4), c0 = PRM(m, 5), sl = PRM(m, 6), G0 = PRM(m, 7);
            double rho = e->rhok, et = 1.0 - r0 / rho, dd = 1.0 - sl * et;
            double ph = r0 * c0 * c0 * et / (dd * dd);
            double dph = r0 * c0 * c0 * (1.0 + sl * et) / (dd * dd * dd);
            double detadrho = r0 / (rho * rho);
            double dp = dph * detadrho;
            double de = (ph + et * dph) / (2.0 * r0) * detadrho;
            return dp - G * rho * de + (e->p * (G + 1.0) - ph) / rho + (4.0 / 3.0) * G0 / rho;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Per-cell operations of BoxAccessCellArray, on a state array X.          */
/* ------------------------------------------------------------------------ */
static void cell_ecell(const tjp_sim* s, const double* X, long N, long c, int m, ecell* e)
{
    const cmap* C = &s->c;
    e->alpha = AT(X, C->ALPHA + m, c);
    e->arho = AT(X, C->ALPHARHO + m, c);
    e->rhok = AT(X, C->RHO_K + m, c);
    e->p = AT(X, C->P, c);
    e->hj2 = C->HJ2 >= 0 ? AT(X, C->HJ2, c) : 0.0;
    e->lam = e->rm0 = e->rm1 = 0.0;
    if (s->p.eos[m] == 4) {
        e->lam = AT(X, C->LAM, c);
        e->rm0 = AT(X, C->RMIX, c);
        e->rm1 = AT(X, C->RMIX + 1, c);
    }
}

static double eff_invG(const tjp_sim* s, const double* X, long N, long c) /* :218-228 */
{
    double tot = 0.0;
    for (int m = 0; m < s->p.M; ++m) {
        ecell e;
        cell_ecell(s, X, N, c, m, &e);
        tot += eos_invG(s, m, &e);
    }
    return tot;
}
static double eff_e_nonthermal(const tjp_sim* s, const double* X, long N, long c) /* :230-240 */
{
    double tot = 0.0;
    for (int m = 0; m < s->p.M; ++m) {
        ecell e;
        cell_ecell(s, X, N, c, m, &e);
        tot += (eos_e_cold(s, m, &e) + eos_e_shear(s, m, &e));
    }
    return tot;
}
static double eff_p_nonthermal(const tjp_sim* s, const double* X, long N, long c) /* :242-252 */
{
    double tot = 0.0;
    for (int m = 0; m < s->p.M; ++m) {
        ecell e;
        cell_ecell(s, X, N, c, m, &e);
        tot += eos_p_cold(s, m, &e) + eos_p_shear(s, m, &e);
    }
    return tot;
}

/* getDeviatoricHenckyStrain + getHenckyJ2 (boxaccesscellarray.cpp:326-380) */
static void hencky(const tjp_sim* s, double* X, long N, long c)
{
    const cmap* C = &s->c;
    int any_solid = 0;
    for (int m = 0; m < s->p.M; ++m)
        if (s->p.phase[m] == 0) any_solid = 1;
    if (!any_solid) return;
    double V[9], B[9], Binv[9], dev[9], prod[9];
    for (int q = 0; q < 9; ++q) V[q] = AT(X, C->V + q, c);
    mmT(V, V, B);
    invert3(B, Binv);
    for (int q = 0; q < 9; ++q) {
        dev[q] = 0.5 * 0.5 * (B[q] - Binv[q]);
        AT(X, C->DEVH + q, c) = dev[q];
    }
    mmT(dev, dev, prod);
    AT(X, C->HJ2, c) = trace3(prod);
}

/* stressTensor (boxaccesscellarray.cpp:176-216) */
static void stress(const tjp_sim* s, double* X, long N, long c)
{
    const cmap* C = &s->c;
    double Gt = 0.0;
    int solid = 0;
    for (int m = 0; m < s->p.M; ++m)
        if (s->p.phase[m] == 0) {
            ecell e;
            cell_ecell(s, X, N, c, m, &e);
            solid = 1;
            Gt += eos_G(s, m, &e) * (eos_invG(s, m, &e));
        }
    Gt = Gt / eff_invG(s, X, N, c);
    double p = AT(X, C->P, c);
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) {
            double dl = (double)(r == q);
            if (solid)
                AT(X, C->SIGMA + 3 * r + q, c) = -p * dl + 2.0 * Gt * AT(X, C->DEVH + 3 * r + q, c);
            else
                AT(X, C->SIGMA + 3 * r + q, c) = -p * dl;
        }
}

/* MixtureEOS root finding (equationofstate.cpp:238-376) for material 0:
 * the mixture densities at which the two components' temperatures agree. */
static double mix_rhob(const tjp_sim* s, double* X, long N, long c, double rhoa) /* rhobFunc :243-246 */
{
    const cmap* C = &s->c;
    return (1.0 - AT(X, C->LAM, c)) / (1.0 / AT(X, C->RHO_K, c) - AT(X, C->LAM, c) / rhoa);
}

static double mix_bisection(const tjp_sim* s, double* X, long N, long c, double rhoTry, double ke) /* :262-272 */
{
    const cmap* C = &s->c;
    AT(X, C->RMIX, c) = rhoTry;
    AT(X, C->RMIX + 1, c) = mix_rhob(s, X, N, c, rhoTry);
    double p = (AT(X, C->E, c) - ke - eff_e_nonthermal(s, X, N, c) + eff_p_nonthermal(s, X, N, c)) / (eff_invG(s, X, N, c));
    /* pressureFunction (:251-260) */
    return ((p - PRM(0, 1)) / (AT(X, C->RMIX, c) * MG1(0) * PRM(0, 3))) -
           ((p - PRM(0, 5)) / (AT(X, C->RMIX + 1, c) * MG2(0) * PRM(0, 7)));
}

static int sgn_d(double v) { return (0.0 < v) - (v < 0.0); }

static void mix_root_find(tjp_sim* s, double* X, long N, long c, double ke) /* rootFind :274-376 */
{
    const cmap* C = &s->c;
    const double lam = AT(X, C->LAM, c), rk = AT(X, C->RHO_K, c);
    if (PRM(0, 1) == 0.0 && PRM(0, 5) == 0.0) {
        AT(X, C->RMIX, c) = rk * (lam + (1.0 - lam) * (MG2(0) * PRM(0, 7)) / (MG1(0) * PRM(0, 3)));
        AT(X, C->RMIX + 1, c) = mix_rhob(s, X, N, c, AT(X, C->RMIX, c));
        return;
    }
    if (lam > 1.0 - 1E-3) {
        AT(X, C->RMIX, c) = rk;
        AT(X, C->RMIX + 1, c) = rk;
        return;
    } else if (lam < 1E-3) {
        AT(X, C->RMIX + 1, c) = rk;
        AT(X, C->RMIX, c) = rk;
        return;
    }
    double A = lam * rk + 1E-10, B = 1000000.0;
    double mid = 0.5 * (A + B);
    if (fabs(mix_bisection(s, X, N, c, A, ke)) <= 1E-4) {
        AT(X, C->RMIX, c) = A;
        AT(X, C->RMIX + 1, c) = mix_rhob(s, X, N, c, AT(X, C->RMIX, c));
        return;
    } else if (fabs(mix_bisection(s, X, N, c, B, ke)) <= 1E-4) {
        AT(X, C->RMIX, c) = B;
        AT(X, C->RMIX + 1, c) = mix_rhob(s, X, N, c, AT(X, C->RMIX, c));
        return;
    }
    if (sgn_d(mix_bisection(s, X, N, c, A, ke)) == sgn_d(mix_bisection(s, X, N, c, B, ke))) {
        s->err = -5; /* "Error in root Bisection" and exit(1) in the reference */
        return;
    }
    for (int n = 0;; n++) {
        if (sgn_d(mix_bisection(s, X, N, c, mid, ke)) == sgn_d(mix_bisection(s, X, N, c, A, ke))) A = mid;
        else B = mid;
        mid = 0.5 * (A + B);
        if (fabs(A - B) / (A + B) < 1E-7) {
            AT(X, C->RMIX, c) = mid;
            AT(X, C->RMIX + 1, c) = mix_rhob(s, X, N, c, AT(X, C->RMIX, c));
            return;
        }
    }
}

/* conservativeToPrimitive (boxaccesscellarray.cpp:67-122) */
static void c2p(const tjp_sim* s, double* X, long N, long c)
{
    const cmap* C = &s->c;
    int M = s->p.M;
    AT(X, C->RHO, c) = 0;
    for (int m = 0; m < M; ++m) {
        AT(X, C->RHO_K + m, c) = AT(X, C->ALPHARHO + m, c) / AT(X, C->ALPHA + m, c);
        AT(X, C->RHO, c) += AT(X, C->ALPHARHO + m, c);
        if (s->p.plastic && s->p.phase[m] == 0) AT(X, C->EPS + m, c) = AT(X, C->ARE + m, c) / AT(X, C->ALPHARHO + m, c);
    }
    hencky(s, X, N, c);
    double ke = 0.0;
    for (int r = 0; r < 3; ++r) {
        AT(X, C->VEL + r, c) = AT(X, C->RHOU + r, c) / AT(X, C->RHO, c);
        ke += 0.5 * AT(X, C->RHO, c) * AT(X, C->VEL + r, c) * AT(X, C->VEL + r, c);
    }
    if (s->p.nmix) { /* :104-113 */
        AT(X, C->LAM, c) = AT(X, C->ARL, c) / AT(X, C->ALPHARHO, c);
        mix_root_find((tjp_sim*)s, X, N, c, ke);
    }
    AT(X, C->P, c) = (AT(X, C->E, c) - ke - eff_e_nonthermal(s, X, N, c) + eff_p_nonthermal(s, X, N, c)) / (eff_invG(s, X, N, c));
    stress(s, X, N, c);
}

/* primitiveToConservative (boxaccesscellarray.cpp:124-174) */
static void p2c(const tjp_sim* s, double* X, long N, long c)
{
    const cmap* C = &s->c;
    int M = s->p.M;
    AT(X, C->RHO, c) = 0;
    for (int m = 0; m < M; ++m) {
        AT(X, C->ALPHARHO + m, c) = AT(X, C->ALPHA + m, c) * AT(X, C->RHO_K + m, c);
        AT(X, C->RHO, c) += AT(X, C->ALPHARHO + m, c);
        if (s->p.nmix && m == 0) {
            AT(X, C->ARL, c) = AT(X, C->LAM, c) * AT(X, C->ALPHA, c) * AT(X, C->RHO_K, c);
            /* defineMixtureDensities (equationofstate.cpp:390-396) */
            const double lam = AT(X, C->LAM, c), pp = AT(X, C->P, c);
            AT(X, C->RMIX, c) = AT(X, C->RHO_K, c) * (lam + (1.0 - lam) * ((pp - PRM(0, 1)) / (pp - PRM(0, 5))) *
                                                               ((PRM(0, 7) * MG2(0)) / (PRM(0, 3) * MG1(0))));
            AT(X, C->RMIX + 1, c) = mix_rhob(s, X, N, c, AT(X, C->RMIX, c));
        }
        if (s->p.plastic && s->p.phase[m] == 0) AT(X, C->ARE + m, c) = AT(X, C->EPS + m, c) * AT(X, C->ALPHARHO + m, c);
    }
    hencky(s, X, N, c);
    double ke = 0.0;
    for (int r = 0; r < 3; ++r) {
        AT(X, C->RHOU + r, c) = AT(X, C->VEL + r, c) * AT(X, C->RHO, c);
        ke += 0.5 * AT(X, C->RHO, c) * AT(X, C->VEL + r, c) * AT(X, C->VEL + r, c);
    }
    AT(X, C->E, c) = AT(X, C->P, c) * eff_invG(s, X, N, c) + eff_e_nonthermal(s, X, N, c) - eff_p_nonthermal(s, X, N, c) + ke;
    stress(s, X, N, c);
}

/* getSoundSpeed (boxaccesscellarray.cpp:254-285) */
static void sound_speed(const tjp_sim* s, double* X, long N, long c)
{
    const cmap* C = &s->c;
    double a = 0.0, xit = 0.0;
    for (int m = 0; m < s->p.M; ++m) {
        ecell e;
        cell_ecell(s, X, N, c, m, &e);
        double v = eos_xi(s, m, &e) * eos_c2(s, m, &e) * AT(X, C->ALPHARHO + m, c) / AT(X, C->RHO, c);
        a += (0.0 < v) ? v : 0.0;
        xit += eos_xi(s, m, &e) * AT(X, C->ALPHA + m, c);
    }
    if (a <= 0.0) a = 1E-6;
    AT(X, C->A, c) = sqrt(a / xit);
}

/* cleanUpAlpha on one cell (boxaccesscellarray.cpp:530-599); returns nonzero
 * on the reference's fatal conditions. */
static int cleanup_alpha_cell(const tjp_sim* s, double* X, long N, long c)
{
    const cmap* C = &s->c;
    double tot = 0.0;
    int nan = 0;
    for (int m = 0; m < s->p.M; ++m) {
        double* a = &AT(X, C->ALPHA + m, c);
        if (isnan(*a)) {
            *a = 0.0;
            if (nan == 0) nan = m;
            else return -3;
        } else if (*a < 0.0) *a = 1E-6;
        else if (*a > 1.0) *a = 1.0;
        tot += *a;
    }
    if (nan > 0) {
        AT(X, C->ALPHA + nan, c) = 1.0 - tot;
        tot += AT(X, C->ALPHA + nan, c);
    }
    if (tot <= 0.0) return -3;
    for (int m = 0; m < s->p.M; ++m) AT(X, C->ALPHA + m, c) *= 1.0 / tot;
    return 0;
}

/* transverseWaveSpeed on a star-state cell (boxaccesscellarray.cpp:287-324) */
static double transverse_speed(const tjp_sim* s, double* X, long N, long c)
{
    const cmap* C = &s->c;
    hencky(s, X, N, c);
    double b = 0.0;
    for (int m = 0; m < s->p.M; ++m)
        if (s->p.phase[m] == 0) {
            ecell e;
            cell_ecell(s, X, N, c, m, &e);
            b += eos_invG(s, m, &e) * eos_G(s, m, &e) / (AT(X, C->RHO_K + m, c));
        }
    if (isnan(b) || b < 0.0) b = 0.0;
    double t = sqrt(b / eff_invG(s, X, N, c));
    if (isnan(t)) t = 0.0;
    return t;
}

/* ------------------------------------------------------------------------ */
/* Riemann solvers (hllc.cpp:1-487, flux.cpp:5-47) on "cells" stored as      */
/* single-cell state vectors (Ncomp doubles, stride 1).                      */
/* ------------------------------------------------------------------------ */
#define CV(x, comp) ((x)[(comp)])

static double pflux(const tjp_sim* s, int comp, const double* U, int d) /* flux.cpp:33-47 */
{
    const cmap* C = &s->c;
    double ud = CV(U, C->VEL + d);
    if (comp >= C->ALPHA && comp < C->ALPHA + s->p.M) return CV(U, comp) * ud;
    if (comp >= C->ALPHARHO && comp < C->ALPHARHO + s->p.M) return CV(U, comp) * ud;
    if (C->ARE >= 0 && comp >= C->ARE && comp < C->ARE + s->p.M) return CV(U, comp) * ud;
    if (comp == C->ARL) return CV(U, comp) * ud;
    if (comp >= C->RHOU && comp < C->RHOU + 3) return CV(U, comp) * ud - CV(U, C->SIGMA + 3 * (comp - C->RHOU) + d);
    if (comp == C->E) {
        double r = 0.0;
        for (int i = 0; i < 3; ++i) r += CV(U, C->VEL + i) * CV(U, C->SIGMA + 3 * i + d);
        return CV(U, C->E) * ud - r;
    }
    /* V_TENSOR */
    int q = comp - C->V, row = q / 3, col = q % 3;
    return CV(U, comp) * ud - CV(U, C->V + 3 * d + col) * CV(U, C->VEL + row);
}

/* getStarState (hllc.cpp:12-73) */
static void star_state(const tjp_sim* s, const double* U, double* Us, double SK, double Ss, int d)
{
    const cmap* C = &s->c;
    const double tol = 1E-20;
    double ud = CV(U, C->VEL + d);
    double mult = (fabs((Ss - ud) / Ss) < tol ? 1.0 : (SK - ud) / (SK - Ss));
    CV(Us, C->RHO) = 0.0;
    for (int m = 0; m < s->p.M; ++m) {
        CV(Us, C->ALPHA + m) = CV(U, C->ALPHA + m);
        CV(Us, C->ALPHARHO + m) = mult * CV(U, C->ALPHARHO + m);
        CV(Us, C->RHO_K + m) = CV(Us, C->ALPHARHO + m) / CV(Us, C->ALPHA + m);
        if (s->p.nmix && m == 0) CV(Us, C->ARL) = mult * CV(U, C->ARL);
        if (s->p.plastic && s->p.phase[m] == 0) CV(Us, C->ARE + m) = mult * CV(U, C->ARE + m);
        CV(Us, C->RHO) += CV(Us, C->ALPHARHO + m);
    }
    for (int row = 0; row < 3; ++row) {
        if (row == d) CV(Us, C->RHOU + row) = mult * CV(U, C->RHO) * Ss;
        else CV(Us, C->RHOU + row) = mult * CV(U, C->RHOU + row);
        CV(Us, C->VEL + row) = CV(Us, C->RHOU + row) / CV(Us, C->RHO);
        if (s->p.solid)
            for (int col = 0; col < 3; ++col) {
                if (row == d) CV(Us, C->V + 3 * row + col) = CV(U, C->V + 3 * row + col);
                else CV(Us, C->V + 3 * row + col) = mult * CV(U, C->V + 3 * row + col);
            }
    }
    CV(Us, C->E) = mult * CV(U, C->RHO) *
                   (CV(U, C->E) / CV(U, C->RHO) +
                    (Ss - ud) * (Ss - (CV(U, C->SIGMA + 4 * d)) / (CV(U, C->RHO) * (SK - ud))));
}

/* getSstar (hllc.cpp:5-8) */
static double sstar(const tjp_sim* s, const double* L, const double* R, double SL, double SR, int d)
{
    const cmap* C = &s->c;
    return (-CV(R, C->SIGMA + 4 * d) + CV(L, C->SIGMA + 4 * d) + CV(L, C->RHOU + d) * (SL - CV(L, C->VEL + d)) -
            CV(R, C->RHOU + d) * (SR - CV(R, C->VEL + d))) /
           (CV(L, C->RHO) * (SL - CV(L, C->VEL + d)) - CV(R, C->RHO) * (SR - CV(R, C->VEL + d)));
}

/* Conservative-variable list (accesspattern.cpp:48-75): alpha, alphaRho, rhoU,
 * E, alphaRhoLambda, V, alphaRhoEpsilon. */
static int cons_list(const tjp_sim* s, int* out)
{
    const cmap* C = &s->c;
    int n = 0;
    for (int m = 0; m < s->p.M; ++m) out[n++] = C->ALPHA + m;
    for (int m = 0; m < s->p.M; ++m) out[n++] = C->ALPHARHO + m;
    for (int r = 0; r < 3; ++r) out[n++] = C->RHOU + r;
    out[n++] = C->E;
    if (s->p.nmix) out[n++] = C->ARL;
    if (s->p.solid)
        for (int q = 0; q < 9; ++q) out[n++] = C->V + q;
    if (s->p.plastic)
        for (int m = 0; m < s->p.M; ++m) out[n++] = C->ARE + m;
    return n;
}

/* Primitive-variable list: alpha, rho_k, u, p, lambda, V, epsilon. */
static int prim_list(const tjp_sim* s, int* out)
{
    const cmap* C = &s->c;
    int n = 0;
    for (int m = 0; m < s->p.M; ++m) out[n++] = C->ALPHA + m;
    for (int m = 0; m < s->p.M; ++m) out[n++] = C->RHO_K + m;
    for (int r = 0; r < 3; ++r) out[n++] = C->VEL + r;
    out[n++] = C->P;
    if (s->p.nmix) out[n++] = C->LAM;
    if (s->p.solid)
        for (int q = 0; q < 9; ++q) out[n++] = C->V + q;
    if (s->p.plastic)
        for (int m = 0; m < s->p.M; ++m) out[n++] = C->EPS + m;
    return n;
}

/* Load the single-cell state of array X at a (possibly ghost) cell. */
static void load_cell(const tjp_sim* s, const pdom* D, const double* X, int i, int j, int k, double* out)
{
    int ijk[3] = {i, j, k}, refl[3];
    map_cell(s, D, ijk, refl);
    long N = D->N, c = lin(D, ijk[0], ijk[1], ijk[2]);
    for (int q = 0; q < s->c.ncomp; ++q) {
        double v = AT(X, q, c);
        out[q] = odd_sign(s, q, refl) < 0.0 ? -v : v;
    }
}

/* HLLC (hllc.cpp:384-487) or 5-wave (hllc.cpp:133-380) flux at one face.
 * L = left state (UR of cell i-1), R = right state (UL of cell i).
 * F receives Ncomp values: the conservative fluxes, USTAR = S*, VSTAR.
 * Returns the star alpha source side: 0 left, 1 right; -2 on NaN speeds. */
static int face_flux(const tjp_sim* s, double* L, double* R, double* F, int d)
{
    const cmap* C = &s->c;
    int nc = C->ncomp;
    double Ls[64], Rs[64], Uss[64];
    int cons[64];
    int ncons = cons_list(s, cons);
    memset(Ls, 0, sizeof Ls);
    memset(Rs, 0, sizeof Rs);
    memset(Uss, 0, sizeof Uss);
    double aL = CV(L, C->VEL + d), aR = CV(R, C->VEL + d);
    double x1 = fabs(aL) + CV(L, C->A), x2 = fabs(aR) + CV(R, C->A);
    double SR = (x1 < x2) ? x2 : x1;
    double SL = -SR;
    double Ss = sstar(s, L, R, SL, SR, d);
    CV(F, C->USTAR) = Ss;
    int side;
    if (!s->p.solid) {
        if (SL >= 0.0) {
            star_state(s, L, Ls, SL, Ss, d);
            for (int q = 0; q < ncons; ++q) {
                int n = cons[q];
                F[n] = (n < C->ALPHA + s->p.M) ? pflux(s, n, Ls, d) : pflux(s, n, L, d);
            }
            side = 0;
        } else if (Ss >= 0.0) {
            star_state(s, L, Ls, SL, Ss, d);
            for (int q = 0; q < ncons; ++q) {
                int n = cons[q];
                F[n] = (n < C->ALPHA + s->p.M) ? pflux(s, n, Ls, d) : pflux(s, n, L, d) + SL * (Ls[n] - L[n]);
            }
            side = 0;
        } else if (SR >= 0.0) {
            star_state(s, R, Rs, SR, Ss, d);
            for (int q = 0; q < ncons; ++q) {
                int n = cons[q];
                F[n] = (n < C->ALPHA + s->p.M) ? pflux(s, n, Rs, d) : pflux(s, n, R, d) + SR * (Rs[n] - R[n]);
            }
            side = 1;
        } else {
            star_state(s, R, Rs, SR, Ss, d);
            for (int q = 0; q < ncons; ++q) {
                int n = cons[q];
                F[n] = (n < C->ALPHA + s->p.M) ? pflux(s, n, Rs, d) : pflux(s, n, R, d);
            }
            side = 1;
        }
        (void)nc;
        return side;
    }

    /* 5-wave solver for solids. */
    if (isnan(SL) || isnan(SR) || isnan(Ss)) return -2;
    double SLT = 0.0, SRT = 0.0;
    const double* vsrc;
    /* Star-state cells keep their own Hencky scratch (transverseWaveSpeed). */
#define TWS(X) transverse_speed(s, (X), 1, 0)
#define STARSTAR(UK, UKs, SKT)                                                                                         \
    do {                                                                                                               \
        for (int q = 0; q < nc; ++q) Uss[q] = UKs[q];                                                                  \
        for (int i = 0; i < 3; ++i)                                                                                    \
            UKs[C->SIGMA + 3 * i + d] =                                                                                \
                (Ls[C->RHO] * (Ss - SLT) * Rs[C->RHO] * (Ss - SRT) * (L[C->VEL + i] - R[C->VEL + i]) +                \
                 Ls[C->RHO] * (Ss - SLT) * R[C->SIGMA + 3 * i + d] - Rs[C->RHO] * (Ss - SRT) * L[C->SIGMA + 3 * i + d]) / \
                (Ls[C->RHO] * (Ss - SLT) - Rs[C->RHO] * (Ss - SRT));                                                   \
        for (int row = 0; row < 3; ++row) {                                                                            \
            if (row == d) continue;                                                                                    \
            Uss[C->RHOU + row] += (UKs[C->SIGMA + 3 * row + d] - UK[C->SIGMA + 3 * row + d]) / (Ss - (SKT));           \
            Uss[C->VEL + row] = Uss[C->RHOU + row] / Uss[C->RHO];                                                      \
        }                                                                                                              \
        for (int row = 0; row < 3; ++row) {                                                                            \
            if (row == d) continue;                                                                                    \
            Uss[C->E] += (Uss[C->VEL + row] * UKs[C->SIGMA + 3 * row + d] - UK[C->VEL + row] * UK[C->SIGMA + 3 * row + d]) / \
                         (Ss - (SKT));                                                                                 \
            for (int col = 0; col < 3; ++col)                                                                          \
                Uss[C->V + 3 * row + col] += (Uss[C->V + 3 * d + col] * (Uss[C->VEL + row] - UK[C->VEL + row])) / (Ss - (SKT)); \
        }                                                                                                              \
    } while (0)

    if (SL >= 0.0) {
        star_state(s, L, Ls, SL, Ss, d);
        for (int q = 0; q < ncons; ++q) {
            int n = cons[q];
            F[n] = (n < C->ALPHA + s->p.M) ? pflux(s, n, Ls, d) : pflux(s, n, L, d);
        }
        vsrc = L;
        side = 0;
    } else if (Ss >= 0.0) {
        star_state(s, L, Ls, SL, Ss, d);
        SLT = Ss - TWS(Ls);
        if (SLT >= 0.0) {
            for (int q = 0; q < ncons; ++q) {
                int n = cons[q];
                F[n] = (n < C->ALPHA + s->p.M) ? pflux(s, n, Ls, d) : pflux(s, n, L, d) + SL * (Ls[n] - L[n]);
            }
            vsrc = Ls;
        } else {
            star_state(s, R, Rs, SR, Ss, d);
            SRT = Ss + TWS(Rs);
            STARSTAR(L, Ls, SLT);
            for (int q = 0; q < ncons; ++q) {
                int n = cons[q];
                F[n] = (n < C->ALPHA + s->p.M) ? pflux(s, n, Ls, d)
                                               : pflux(s, n, L, d) + SL * (Ls[n] - L[n]) + SLT * (Uss[n] - Ls[n]);
            }
            vsrc = Uss;
        }
        side = 0;
    } else if (SR >= 0.0) {
        star_state(s, R, Rs, SR, Ss, d);
        SRT = Ss + TWS(Rs);
        if (SRT >= 0.0) {
            star_state(s, L, Ls, SL, Ss, d);
            SLT = Ss - TWS(Ls);
            STARSTAR(R, Rs, SRT);
            for (int q = 0; q < ncons; ++q) {
                int n = cons[q];
                F[n] = (n < C->ALPHA + s->p.M) ? pflux(s, n, Rs, d)
                                               : pflux(s, n, R, d) + SR * (Rs[n] - R[n]) + SRT * (Uss[n] - Rs[n]);
            }
            vsrc = Uss;
        } else {
            for (int q = 0; q < ncons; ++q) {
                int n = cons[q];
                F[n] = (n < C->ALPHA + s->p.M) ? pflux(s, n, Rs, d) : pflux(s, n, R, d) + SR * (Rs[n] - R[n]);
            }
            vsrc = Rs;
        }
        side = 1;
    } else {
        star_state(s, R, Rs, SR, Ss, d);
        for (int q = 0; q < ncons; ++q) {
            int n = cons[q];
            F[n] = (n < C->ALPHA + s->p.M) ? pflux(s, n, Rs, d) : pflux(s, n, R, d);
        }
        vsrc = R;
        side = 1;
    }
    for (int q = 0; q < 9; ++q) F[C->VSTAR + q] = vsrc[C->V + q];
    if (isnan(SL) || isnan(SR) || isnan(Ss) || isnan(SLT) || isnan(SRT)) return -2;
#undef TWS
#undef STARSTAR
    return side;
}

/* ------------------------------------------------------------------------ */
/* One RK stage: HLLCadvance (hllc.cpp:579-695), U -> U1.                   */
/* ------------------------------------------------------------------------ */
static double vanleer(double r) /* hllc.cpp:527-537 */
{
    if (r <= 0.0) return 0.0;
    double a = 2.0 / (1.0 + r), b = 2.0 * r / (1.0 + r);
    return (b < a) ? b : a;
}

static double sgn(double v) { return (double)((0.0 < v) - (v < 0.0)); }

static int box_contains(const int* b, int i, int j, int k)
{
    return i >= b[0] && i <= b[3] && j >= b[1] && j <= b[4] && k >= b[2] && k <= b[5];
}

static long face_lin(const pdom* D, int d, int i, int j, int k)
{
    int nf0 = D->n[0] + (d == 0), nf1 = D->n[1] + (d == 1);
    return i + (long)nf0 * (j + (long)nf1 * k);
}

/* Young's normal component (thinc.cpp:28-53), 2-D only. */
static double youngs(const tjp_sim* s, const pdom* D, const double* U, int m, int i, int j, int k, int d)
{
    int a = s->c.ALPHA + m;
#define NB(di, dj) gv(s, D, U, a, i + (di), j + (dj), k)
    double nx = -1.0 / (8.0 * D->dx[0]) *
                (NB(1, 1) + 2.0 * NB(1, 0) + NB(1, -1) - NB(-1, 1) - 2.0 * NB(-1, 0) - NB(-1, -1));
    double ny = -1.0 / (8.0 * D->dx[1]) *
                (NB(1, 1) + 2.0 * NB(0, 1) + NB(-1, 1) - NB(-1, -1) - 2.0 * NB(0, -1) - NB(1, -1));
#undef NB
    double norm = sqrt(nx * nx + ny * ny);
    if (norm < 1E-20) return 0;
    return d == 0 ? fabs(nx / norm) : fabs(ny / norm);
}

static int stage(tjp_sim* s, pdom* D, double* U, double* U1, double dt)
{
    const cmap* C = &s->c;
    const int M = s->p.M, nc = C->ncomp;
    const long N = D->N;
    int prims[64], cons[64];
    int nprim = prim_list(s, prims), ncons = cons_list(s, cons);
    int err = 0;

    memcpy(U1, U, sizeof(double) * nc * N); /* U1 = U (hllc.cpp:583) */
    for (int d = 0; d < s->p.dim; ++d) {
        memcpy(D->UL, U, sizeof(double) * nc * N); /* UL = U; UR = U (589-590) */
        memcpy(D->UR, U, sizeof(double) * nc * N);
        int off[3] = {0, 0, 0};
        off[d] = 1;

        /* MUSCL extrapolation (hllc.cpp:541-575). */
        if (s->p.muscl) {
#pragma omp parallel for schedule(static)
            for (long c = 0; c < N; ++c) {
                int i = (int)(c % D->n[0]), j = (int)((c / D->n[0]) % D->n[1]), k = (int)(c / ((long)D->n[0] * D->n[1]));
                for (int q = 0; q < nprim; ++q) {
                    int n = prims[q];
                    double u0 = AT(U, n, c);
                    double um = gv(s, D, U, n, i - off[0], j - off[1], k - off[2]);
                    double up = gv(s, D, U, n, i + off[0], j + off[1], k + off[2]);
                    double r = (u0 - um) / (up - u0);
                    if (isinf(r) || isnan(r)) r = 0.0;
                    double grad = vanleer(r) * 0.5 * (up - um);
                    AT(D->UL, n, c) = u0 - 0.5 * grad;
                    AT(D->UR, n, c) = u0 + 0.5 * grad;
                }
            }
        }

        /* BVD-THINC (thinc.cpp:67-208), with the reference's scratch history:
         * candidates written into the persistent ULStar/URStar alpha at mixed
         * cells, neighbour reads from the same box or its ghost cells. */
        if (s->p.thinc) {
            const double beta0 = s->p.thinc_beta, eps = 1E-20;
#pragma omp parallel for schedule(static)
            for (long c = 0; c < N; ++c) {
                int i = (int)(c % D->n[0]), j = (int)((c / D->n[0]) % D->n[1]), k = (int)(c / ((long)D->n[0] * D->n[1]));
                D->flag[c] = 0;
                for (int m = 0; m < M; ++m) {
                    int a = C->ALPHA + m;
                    double aL = gv(s, D, U, a, i - off[0], j - off[1], k - off[2]);
                    double aR = gv(s, D, U, a, i + off[0], j + off[1], k + off[2]);
                    double a0 = AT(U, a, c);
                    double mn = (aR < aL) ? aR : aL;
                    double mx = ((aL < aR) ? aR : aL) - mn;
                    double theta = sgn(aR - aL);
                    double Cc = (mx < eps) ? 0.0 : (a0 - mn + eps) / (mx + eps);
                    double delta = 1E-4;
                    int mixed = (Cc > delta) && (Cc < (0.999999 - delta)) && ((aR - a0) * (a0 - aL) >= 0.0);
                    D->flag[c] = (unsigned char)mixed;
                    D->mixed[(size_t)m * N + c] = (unsigned char)mixed;
                    if (mixed) {
                        double nvc = (s->p.dim == 2) ? youngs(s, D, U, m, i, j, k, d) : 1.0;
                        double beta = nvc * beta0 + 0.01;
                        double coshB = tjm_cosh(beta), tanhB = tjm_tanh(beta);
                        double B = tjm_exp(theta * beta * ((2.0 * Cc) - 1.0));
                        double A = ((B / coshB) - 1.0) / tanhB;
                        D->urstar[(size_t)m * N + c] = mn + (mx / 2.0) * (1.0 + theta * ((tanhB + A) / (1.0 + A * tanhB)));
                        D->ulstar[(size_t)m * N + c] = mn + (mx / 2.0) * (1.0 + theta * A);
                    }
                }
            }
#pragma omp parallel for schedule(static)
            for (long c = 0; c < N; ++c) {
                int i = (int)(c % D->n[0]), j = (int)((c / D->n[0]) % D->n[1]), k = (int)(c / ((long)D->n[0] * D->n[1]));
                const int* bx = D->box + 6 * D->cell_box[c];
                int im = i - off[0], jm = j - off[1], km = k - off[2];
                int ip = i + off[0], jp = j + off[1], kp = k + off[2];
                int in_m = box_contains(bx, im, jm, km), in_p = box_contains(bx, ip, jp, kp);
                for (int m = 0; m < M; ++m) {
                    int a = C->ALPHA + m;
                    /* UR.left and UL.right: this pass's MUSCL value inside the
                     * box, the stage input in a ghost (hllc.cpp:589-590). */
                    double urm = in_m ? AT(D->UR, a, lin(D, im, jm, km)) : gv(s, D, U, a, im, jm, km);
                    double ulp = in_p ? AT(D->UL, a, lin(D, ip, jp, kp)) : gv(s, D, U, a, ip, jp, kp);
                    /* UTHINC_R.left: URStar ghosts are never written (0).
                     * UTHINC_L.right: ULStar's ghost at hi+1 holds the star
                     * alpha of the last flux pass along d. */
                    double trm = in_m ? D->urstar[(size_t)m * N + lin(D, im, jm, km)] : 0.0;
                    double tlp = in_p ? D->ulstar[(size_t)m * N + lin(D, ip, jp, kp)]
                                      : D->gstar[d][(size_t)m * D->nf[d] + face_lin(D, d, ip, jp, kp)];
                    double upl = AT(D->UL, a, c), upr = AT(D->UR, a, c);
                    double tpl = D->ulstar[(size_t)m * N + c], tpr = D->urstar[(size_t)m * N + c];
#define TBV(PL, PR)                                                                                                   \
    fmin2(fmin2(fabs(urm - (PL)) + fabs((PR)-ulp), fabs(trm - (PL)) + fabs((PR)-tlp)),                                 \
          fmin2(fabs(urm - (PL)) + fabs((PR)-tlp), fabs(trm - (PL)) + fabs((PR)-ulp)))
#define fmin2(x, y) (((y) < (x)) ? (y) : (x))
                    double tbvm = TBV(upl, upr);
                    double tbvt = TBV(tpl, tpr);
#undef TBV
#undef fmin2
                    D->tbv[(size_t)m * N + c] = (unsigned char)(D->flag[c] && tbvt < tbvm);
                }
            }
#pragma omp parallel for schedule(static)
            for (long c = 0; c < N; ++c)
                for (int m = 0; m < M; ++m)
                    if (D->tbv[(size_t)m * N + c]) {
                        AT(D->UL, C->ALPHA + m, c) = D->ulstar[(size_t)m * N + c];
                        AT(D->UR, C->ALPHA + m, c) = D->urstar[(size_t)m * N + c];
                    }
        }

        /* cleanUpAlpha of UL/UR inside the box loop (hllc.cpp:628-629): box b
         * is cleaned nbox-b times in all, primitiveToConservative and
         * getSoundSpeed (634-638) see it after the first. */
#pragma omp parallel for schedule(static)
        for (long c = 0; c < N; ++c) {
            int reps = s->p.thinc ? D->nbox - D->cell_box[c] : 0;
            for (int side = 0; side < 2; ++side) {
                double* X = side ? D->UR : D->UL;
                if (reps > 0) {
                    int e = cleanup_alpha_cell(s, X, N, c);
                    if (e) err = e;
                }
                p2c(s, X, N, c);
                sound_speed(s, X, N, c);
                for (int r = 1; r < reps; ++r) {
                    double before[TJP_MAX_MAT];
                    for (int m = 0; m < M; ++m) before[m] = AT(X, C->ALPHA + m, c);
                    int e = cleanup_alpha_cell(s, X, N, c);
                    if (e) err = e;
                    int same = 1;
                    for (int m = 0; m < M; ++m) same &= (memcmp(&before[m], &AT(X, C->ALPHA + m, c), sizeof(double)) == 0);
                    if (same) break;
                }
            }
        }

        /* Fluxes on faces lo..hi+1 along d (calc_fluxes / calc_5Wave_fluxes);
         * the left state is UR of cell i-1, the right state UL of cell i, with
         * ghost images at the domain boundary (hllc.cpp:642-646). */
        int nf[3] = {D->n[0], D->n[1], D->n[2]};
        nf[d] += 1;
        long NF = (long)nf[0] * nf[1] * nf[2];
#pragma omp parallel for schedule(static)
        for (long f = 0; f < NF; ++f) {
            int i = (int)(f % nf[0]), j = (int)((f / nf[0]) % nf[1]), k = (int)(f / ((long)nf[0] * nf[1]));
            double L[64], R[64], F[64];
            load_cell(s, D, D->UR, i - off[0], j - off[1], k - off[2], L);
            load_cell(s, D, D->UL, i, j, k, R);
            memset(F, 0, sizeof F);
            int side = face_flux(s, L, R, F, d);
            if (side < 0) { err = side; continue; }
            double* Fd = D->flux[d];
            for (int q = 0; q < nc; ++q) Fd[(size_t)q * NF + f] = F[q];
            if (s->p.thinc) {
                const double* src = side ? R : L;
                int idx[3] = {i, j, k};
                /* ULStar alpha at cell i (a valid cell) or at the ghost i = hi+1 */
                if (idx[d] < D->n[d]) {
                    long c = lin(D, i, j, k);
                    for (int m = 0; m < M; ++m) D->ulstar[(size_t)m * N + c] = src[C->ALPHA + m];
                }
                /* ghost hi+1 of the box to the face's left, if the face is its hi face */
                int lc[3] = {i - off[0], j - off[1], k - off[2]};
                if (lc[d] >= 0) {
                    int b = D->cell_box[lin(D, lc[0], lc[1], lc[2])];
                    if (D->box[6 * b + 3 + d] == lc[d])
                        for (int m = 0; m < M; ++m) D->gstar[d][(size_t)m * D->nf[d] + f] = src[C->ALPHA + m];
                }
            }
        }

        /* update (hllc.cpp:493-523) */
        double dtdx = dt / D->dx[d];
#pragma omp parallel for schedule(static)
        for (long c = 0; c < N; ++c) {
            int i = (int)(c % D->n[0]), j = (int)((c / D->n[0]) % D->n[1]), k = (int)(c / ((long)D->n[0] * D->n[1]));
            long f0 = face_lin(D, d, i, j, k), f1 = face_lin(D, d, i + off[0], j + off[1], k + off[2]);
            const double* Fd = D->flux[d];
#define FL(q, f) Fd[(size_t)(q) * NF + (f)]
            for (int q = 0; q < ncons; ++q) {
                int n = cons[q];
                if (n < C->ALPHA + M)
                    AT(U1, n, c) += dtdx * (FL(n, f0) - FL(n, f1) - AT(U, n, c) * (FL(C->USTAR, f0) - FL(C->USTAR, f1)));
                else if (s->p.solid && n >= C->V && n < C->V + 9) {
                    int row = (n - C->V) / 3, col = (n - C->V) % 3;
                    AT(U1, n, c) += dtdx * (FL(n, f0) - FL(n, f1) - (2.0 / 3.0) * AT(U, n, c) * (FL(C->USTAR, f0) - FL(C->USTAR, f1)) +
                                            AT(U, C->VEL + row, c) * (FL(C->VSTAR + 3 * d + col, f0) - FL(C->VSTAR + 3 * d + col, f1)));
                } else
                    AT(U1, n, c) += dtdx * (FL(n, f0) - FL(n, f1));
            }
#undef FL
        }
    }
    /* U1.conservativeToPrimitive (hllc.cpp:689) */
#pragma omp parallel for schedule(static)
    for (long c = 0; c < N; ++c) c2p(s, U1, N, c);
    return err;
}

/* ------------------------------------------------------------------------ */
/* Plastic radial return (plastic.cpp:76-244) and cleanUpV (:476-528).      */
/* ------------------------------------------------------------------------ */
static int plastic_cell(tjp_sim* s, double* X, long N, long c)
{
    const cmap* C = &s->c;
    int M = s->p.M;
    double tsolid = 0.0;
    for (int m = 0; m < M; ++m)
        if (s->p.phase[m] == 0) tsolid += AT(X, C->ALPHA + m, c);
    if (tsolid <= 0.5) { /* cellIsMostlyFluid */
        for (int m = 0; m < M; ++m) { AT(X, C->EPS + m, c) = 0.0; AT(X, C->ARE + m, c) = 0.0; }
        return 0;
    }
    hencky(s, X, N, c);
    double JT = 0.0, JB = 0.0, norm = 0.0, J, Jn;
    for (int m = 0; m < M; ++m) {
        ecell e;
        cell_ecell(s, X, N, c, m, &e);
        if (s->p.phase[m] == 0) {
            J = sqrt(AT(X, C->HJ2, c));
            double G = eos_G(s, m, &e);
            if (G * J * sqrt(3.0) > s->p.yield_stress[m]) Jn = s->p.yield_stress[m] / (sqrt(3.0) * G);
            else Jn = J;
            AT(X, C->EPS + m, c) += sqrt(2.0 / 3.0) * (J - Jn);
            AT(X, C->ARE + m, c) = AT(X, C->EPS + m, c) * AT(X, C->ALPHARHO + m, c);
        } else {
            J = 0.0;
            Jn = 0.0;
            AT(X, C->EPS + m, c) = 0.0;
            AT(X, C->ARE + m, c) = 0.0;
        }
        JB += (eos_invG(s, m, &e)) * J;
        JT += (eos_invG(s, m, &e)) * Jn;
        norm += (eos_invG(s, m, &e));
    }
    JB *= 1.0 / norm;
    JT *= 1.0 / norm;
    if (JB == 0.0 && JT == 0.0) { JB = 1.0; JT = 1.0; }
    double t1[9], t2[9], t2i[9], Vn[9];
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) {
            double* dv = &AT(X, C->DEVH + 3 * r + q, c);
            if (*dv != 0.0 && JB == 0.0 && JT != 0.0) return -4;
            *dv *= JT / JB;
            t1[3 * r + q] = (double)(r == q) + 0.5 * *dv;
            t2[3 * r + q] = (double)(r == q) - 0.5 * *dv;
        }
    invert3(t2, t2i);
    mm(t2i, t1, Vn);
    for (int q = 0; q < 9; ++q) AT(X, C->V + q, c) = Vn[q];
    return 0;
}

static void cleanup_v_cell(tjp_sim* s, double* X, long N, long c)
{
    const cmap* C = &s->c;
    double ta = 0.0, ts = 0.0;
    for (int m = 0; m < s->p.M; ++m) {
        ta += AT(X, C->ALPHA + m, c);
        if (s->p.phase[m] == 0) ts += AT(X, C->ALPHA + m, c);
    }
    double V[9], B[9], Sq[9];
    for (int q = 0; q < 9; ++q) V[q] = AT(X, C->V + q, c);
    mmT(V, V, B);
    sqrtm3(B, Sq);
    double norm = tjm_pow(det3(Sq), -1.0 / 3.0);
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q)
            AT(X, C->V + 3 * r + q, c) = ((Sq[3 * r + q] * norm * ts) + (double)(r == q) * (ta - ts)) / ta;
}

/* ------------------------------------------------------------------------ */
/* Public API.                                                               */
/* ------------------------------------------------------------------------ */
tjp_sim* tjp_create(const tjp_params* p, int ndomains, const int* n_cells, const double* dim_l, const int* nbox,
                    const int* boxes)
{
    /* THINC exists for 1-D and 2-D only (thinc.cpp:116-127) and reads the
     * MUSCL states it is compared against. */
    if (p->thinc && (p->dim == 3 || !p->muscl)) return NULL;
    if (p->M > TJP_MAX_MAT) return NULL;
    tjp_sim* s = (tjp_sim*)calloc(1, sizeof(tjp_sim));
    s->p = *p;
    s->c = make_cmap(p);
    s->ndom = ndomains;
    s->d = (pdom*)calloc(ndomains, sizeof(pdom));
    const int* bp = boxes;
    int nc = s->c.ncomp;
    for (int q = 0; q < ndomains; ++q) {
        pdom* D = &s->d[q];
        D->N = 1;
        for (int d = 0; d < 3; ++d) {
            D->n[d] = n_cells[3 * q + d];
            D->dx[d] = dim_l[3 * q + d] / (double)D->n[d];
            D->N *= D->n[d];
        }
        D->nbox = nbox[q];
        D->box = (int*)malloc(sizeof(int) * 6 * D->nbox);
        memcpy(D->box, bp, sizeof(int) * 6 * D->nbox);
        bp += 6 * D->nbox;
        D->cell_box = (int*)malloc(sizeof(int) * D->N);
        for (int b = 0; b < D->nbox; ++b) {
            const int* B = D->box + 6 * b;
            for (int k = B[2]; k <= B[5]; ++k)
                for (int j = B[1]; j <= B[4]; ++j)
                    for (int i = B[0]; i <= B[3]; ++i) D->cell_box[lin(D, i, j, k)] = b;
        }
        size_t sz = sizeof(double) * nc * D->N;
        D->U1 = (double*)calloc(1, sz);
        D->U = (double*)calloc(1, sz);
        D->U2 = (double*)calloc(1, sz);
        D->UL = (double*)calloc(1, sz);
        D->UR = (double*)calloc(1, sz);
        for (int d = 0; d < 3; ++d) {
            int nf[3] = {D->n[0], D->n[1], D->n[2]};
            nf[d] += 1;
            D->nf[d] = (long)nf[0] * nf[1] * nf[2];
            D->flux[d] = (double*)calloc((size_t)nc * D->nf[d], sizeof(double));
            D->gstar[d] = (double*)calloc((size_t)p->M * D->nf[d], sizeof(double));
        }
        D->ulstar = (double*)calloc((size_t)p->M * D->N, sizeof(double));
        D->urstar = (double*)calloc((size_t)p->M * D->N, sizeof(double));
        D->mixed = (unsigned char*)calloc((size_t)p->M * D->N, 1);
        D->tbv = (unsigned char*)calloc((size_t)p->M * D->N, 1);
        D->flag = (unsigned char*)calloc(D->N, 1);
    }
    return s;
}

void tjp_destroy(tjp_sim* s)
{
    if (!s) return;
    for (int q = 0; q < s->ndom; ++q) {
        pdom* D = &s->d[q];
        free(D->box); free(D->cell_box); free(D->U1); free(D->U); free(D->U2); free(D->UL); free(D->UR);
        for (int d = 0; d < 3; ++d) { free(D->flux[d]); free(D->gstar[d]); }
        free(D->ulstar); free(D->urstar); free(D->mixed); free(D->tbv); free(D->flag);
    }
    free(s->d);
    free(s);
}

int tjp_set_primitive(tjp_sim* s, int dom, const double* prim)
{
    pdom* D = &s->d[dom];
    const cmap* C = &s->c;
    long N = D->N;
    int M = s->p.M, q = 0;
    for (int m = 0; m < M; ++m, ++q) memcpy(&AT(D->U1, C->ALPHA + m, 0), prim + (size_t)q * N, sizeof(double) * N);
    for (int m = 0; m < M; ++m, ++q) memcpy(&AT(D->U1, C->RHO_K + m, 0), prim + (size_t)q * N, sizeof(double) * N);
    for (int r = 0; r < 3; ++r, ++q) memcpy(&AT(D->U1, C->VEL + r, 0), prim + (size_t)q * N, sizeof(double) * N);
    memcpy(&AT(D->U1, C->P, 0), prim + (size_t)q * N, sizeof(double) * N);
    ++q;
    if (s->p.solid)
        for (int r = 0; r < 9; ++r, ++q) memcpy(&AT(D->U1, C->V + r, 0), prim + (size_t)q * N, sizeof(double) * N);
    if (s->p.plastic)
        for (int m = 0; m < M; ++m, ++q) memcpy(&AT(D->U1, C->EPS + m, 0), prim + (size_t)q * N, sizeof(double) * N);
    if (s->p.nmix) { /* initialise.cpp:66-71 */
        memcpy(&AT(D->U1, C->LAM, 0), prim + (size_t)q * N, sizeof(double) * N);
        memcpy(&AT(D->U1, C->RMIX, 0), &AT(D->U1, C->RHO_K, 0), sizeof(double) * N);
        memcpy(&AT(D->U1, C->RMIX + 1, 0), &AT(D->U1, C->RHO_K, 0), sizeof(double) * N);
    }
    for (long c = 0; c < N; ++c) p2c(s, D->U1, N, c);
    return 0;
}

int tjp_get_state(tjp_sim* s, int dom, double* out)
{
    pdom* D = &s->d[dom];
    memcpy(out, D->U1, sizeof(double) * s->c.ncomp * D->N);
    return 0;
}

int tjp_set_state(tjp_sim* s, int dom, const double* in)
{
    pdom* D = &s->d[dom];
    memcpy(D->U1, in, sizeof(double) * s->c.ncomp * D->N);
    return 0;
}

/* TimeStep::getTimeStep (timestep.cpp:7-70) over one domain. */
static double domain_dt(tjp_sim* s, pdom* D)
{
    const cmap* C = &s->c;
    long N = D->N;
    double dtmin = 1.79769313486231570815e+308;
#pragma omp parallel for schedule(static) reduction(min : dtmin)
    for (long c = 0; c < N; ++c) {
        sound_speed(s, D->U1, N, c);
        for (int n = 0; n < s->p.dim; ++n) {
            double v = D->dx[n] / (AT(D->U1, C->A, c) + fabs(AT(D->U1, C->VEL + n, c)));
            if (v < dtmin) dtmin = v;
        }
    }
    return s->p.cfl * dtmin;
}

/* addGeometricSourceTerm (radial.cpp:5-31) on one cell: every conservative
 * variable gains dt * (multiplier / r) * geometricFlux (flux.cpp:51-77), with
 * r = (i + 0.5) dx[0] and multiplier -2 in 1-D (spherical), -1 otherwise
 * (cylindrical). The fluxes read the velocity and the stress the state holds,
 * which the loop over the conservative variables does not change. */
static void radial_cell(tjp_sim* s, const pdom* D, double* X, long N, long c, double dt)
{
    const cmap* C = &s->c;
    const int M = s->p.M;
    const int i = (int)(c % D->n[0]);
    const double mult = (s->p.dim == 1 ? -2.0 : -1.0);
    const double inv_r = mult / (((double)i + 0.5) * D->dx[0]);
    const double u = AT(X, C->VEL, c);
#define SG(r, q) AT(X, C->SIGMA + 3 * (r) + (q), c)
    for (int m = 0; m < M; ++m) AT(X, C->ALPHA + m, c) += dt * inv_r * 0.0;
    for (int m = 0; m < M; ++m) AT(X, C->ALPHARHO + m, c) += dt * inv_r * (AT(X, C->ALPHARHO + m, c) * u);
    AT(X, C->RHOU + 0, c) += dt * inv_r * (AT(X, C->RHOU + 0, c) * u - SG(0, 0) + SG(2, 2));
    AT(X, C->RHOU + 1, c) += dt * inv_r * (AT(X, C->RHOU + 1, c) * u - SG(0, 1));
    AT(X, C->RHOU + 2, c) += dt * inv_r * (-2.0 * SG(0, 2));
    double vds = 0.0; /* vdotsigma (flux.cpp:19-29) along x */
    for (int r = 0; r < 3; ++r) vds += AT(X, C->VEL + r, c) * SG(r, 0);
    AT(X, C->E, c) += dt * inv_r * (AT(X, C->E, c) * u - vds);
    if (s->p.nmix) AT(X, C->ARL, c) += dt * inv_r * (AT(X, C->ARL, c) * u);
    if (s->p.solid) {
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) {
                double* v = &AT(X, C->V + 3 * r + q, c);
                const double g = (r < 2) ? (1.0 / 3.0) * *v * u : -(2.0 / 3.0) * *v * u;
                *v += dt * inv_r * g;
            }
        if (s->p.plastic)
            for (int m = 0; m < M; ++m) AT(X, C->ARE + m, c) += dt * inv_r * (AT(X, C->ARE + m, c) * u);
    }
#undef SG
}

/* pressureBased_UpdateMassFraction (reactive.cpp:3-26) for material 0:
 * alphaRhoLambda after one explicit Euler step of the pressure-based rate. */
static double reactive_euler(double arl, double arho, double p, double alpha, double dt)
{
    const double sigma = 20.0, nu = 0.5, n = 1.2;
    if (alpha < 0.5) return arl;
    double r = arl - (dt) * (sigma * tjm_pow(arho, 1.0 - nu) * tjm_pow(arl, nu) * tjm_pow((p / 1E6), n));
    if (r < 0.0) r = 0.0;
    return r;
}

/* reactiveUpdate (reactive.cpp:60-103) on one cell: two Euler steps from the
 * same alphaRho, pressure and alpha, averaged with the start value, then
 * conservativeToPrimitive. */
static void reactive_cell(tjp_sim* s, double* X, long N, long c, double dt)
{
    const cmap* C = &s->c;
    const double a0 = AT(X, C->ARL, c), arho = AT(X, C->ALPHARHO, c), p = AT(X, C->P, c), al = AT(X, C->ALPHA, c);
    const double a1 = reactive_euler(a0, arho, p, al, dt);
    const double a2 = reactive_euler(a1, arho, p, al, dt);
    AT(X, C->ARL, c) = ((a0 * (1.0 / 2.0)) + (a2 * (1.0 / 2.0)));
    c2p(s, X, N, c);
}

int tjp_run(tjp_sim* s, double final_t, int max_steps, double* dts, double* t_out)
{
    const cmap* C = &s->c;
    int nc = C->ncomp;
    double t = 0.0;
    int n = 0;
    double dt = 0.0;
    for (; t < final_t && n < max_steps; t += dt, n++) {
        dt = 1.79769313486231570815e+308;
        for (int q = 0; q < s->ndom; ++q) {
            double d = domain_dt(s, &s->d[q]);
            dt = (d < dt ? d : dt);
        }
        if (t + dt > final_t) dt = final_t - t;
        if (n < 5) dt *= 0.2;
        dts[n] = dt;
        for (int q = 0; q < s->ndom; ++q) {
            pdom* D = &s->d[q];
            long N = D->N;
            memcpy(D->U, D->U1, sizeof(double) * nc * N);
            int e = stage(s, D, D->U, D->U1, dt);
            if (!e) e = s->err;
            if (!e) e = stage(s, D, D->U1, D->U2, dt);
            if (!e) e = s->err;
            if (e) { *t_out = t; return e; }
            /* U1 = U*0.5 + U2*0.5 over every component (hllc.cpp:705) */
#pragma omp parallel for schedule(static)
            for (long x = 0; x < (long)nc * N; ++x) D->U1[x] = (D->U[x] * (1.0 / 2.0)) + (D->U2[x] * (1.0 / 2.0));
            if (s->p.reactive && s->p.nmix) { /* main.cpp:149-152 */
#pragma omp parallel for schedule(static)
                for (long c = 0; c < N; ++c) reactive_cell(s, D->U1, N, c, dt);
                if (s->err) { *t_out = t; return s->err; }
            }
            int perr = 0;
            if (s->p.plastic) {
#pragma omp parallel for schedule(static)
                for (long c = 0; c < N; ++c) {
                    int e2 = plastic_cell(s, D->U1, N, c);
                    if (e2) perr = e2;
                    c2p(s, D->U1, N, c);
                }
            }
            if (perr || s->err) { *t_out = t; return perr ? perr : s->err; }
            if (s->p.radial) { /* geometricSourceTerm (radial.cpp:37-54, main.cpp:159-161) */
#pragma omp parallel for schedule(static)
                for (long c = 0; c < N; ++c) {
                    radial_cell(s, D, D->U1, N, c, dt);
                    c2p(s, D->U1, N, c);
                }
                if (s->err) { *t_out = t; return s->err; }
            }
            if (s->p.solid) {
#pragma omp parallel for schedule(static)
                for (long c = 0; c < N; ++c) cleanup_v_cell(s, D->U1, N, c);
            }
            int cerr = 0;
#pragma omp parallel for schedule(static)
            for (long c = 0; c < N; ++c) {
                int e2 = cleanup_alpha_cell(s, D->U1, N, c);
                if (e2) cerr = e2;
            }
            if (cerr) { *t_out = t; return cerr; }
            /* contains_nan (cellarray.cpp:101-116): the result of the last box
             * in MFIter order, over the conservative then primitive lists. */
            int cons[64], prims[64], nan = 0;
            int ncons = cons_list(s, cons), nprim = prim_list(s, prims);
            const int* lb = D->box + 6 * (D->nbox - 1);
            for (int k = lb[2]; k <= lb[5]; ++k)
                for (int j = lb[1]; j <= lb[4]; ++j)
                    for (int i = lb[0]; i <= lb[3]; ++i) {
                        long c = lin(D, i, j, k);
                        for (int q2 = 0; q2 < ncons; ++q2) nan |= isnan(AT(D->U1, cons[q2], c));
                        for (int q2 = 0; q2 < nprim; ++q2) nan |= isnan(AT(D->U1, prims[q2], c));
                    }
            if (nan) { *t_out = t + dt; return -1; }
        }
    }
    *t_out = t;
    return n;
}
