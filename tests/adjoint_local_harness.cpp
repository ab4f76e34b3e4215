// Host build of the local adjoint operators (tenjin_gb300/csrc/tj_adjoint_local.h)
// for the finite-difference checks in test_adjoint_local_cpu.py. Each struct
// is passed as a flat array of doubles in its declaration order.
#include <cmath>

#include "tj_adjoint_local.h"

using namespace tja;

static Eos eos_of(int M, const double* e)
{
    Eos E;
    E.M = M;
    for (int m = 0; m < MM; ++m) {
        E.G[m] = e[m];
        E.pr[m] = e[MM + m];
        E.er[m] = e[2 * MM + m];
    }
    return E;
}

static void put_grad(const GradEos& g, double* out)
{
    for (int m = 0; m < MM; ++m) {
        out[m] += g.G[m];
        out[MM + m] += g.pr[m];
        out[2 * MM + m] += g.er[m];
    }
}

static double ch(double x) { return std::cosh(x); }
static double th(double x) { return std::tanh(x); }
static double ex(double x) { return std::exp(x); }

extern "C" {

void h_cleanup(int M, const double* a, double* out) { cleanup_fwd(M, a, out); }
void h_cleanup_rev(int M, const double* a, const double* l, double* li) { cleanup_rev(M, a, l, li); }

void h_face_state(int M, const double* e, const double* x, int clean, double* out)
{
    face_state_fwd(eos_of(M, e), *(const Prim*)x, clean != 0, *(FS*)out);
}

void h_face_state_rev(int M, const double* e, const double* x, int clean, const double* l, double* lx, double* ge)
{
    GradEos g;
    zero(g);
    Prim r;
    zero(r);
    face_state_rev(eos_of(M, e), *(const Prim*)x, clean != 0, *(const FS*)l, r, g);
    *(Prim*)lx = r;
    put_grad(g, ge);
}

int h_hllc(int M, const double* L, const double* R, int d, double* out)
{
    HllcOut o;
    hllc_fwd(M, *(const FS*)L, *(const FS*)R, d, o);
    double* p = out;
    for (int m = 0; m < MM; ++m) *p++ = m < M ? o.Fa[m] : 0.0;
    for (int m = 0; m < MM; ++m) *p++ = m < M ? o.Far[m] : 0.0;
    *p++ = o.Fru[0];
    *p++ = o.Fru[1];
    *p++ = o.FE;
    *p++ = o.Ss;
    return o.side;
}

void h_hllc_rev(int M, const double* L, const double* R, int d, const double* lf, double* lL, double* lR)
{
    HllcOut l;
    const double* p = lf;
    for (int m = 0; m < MM; ++m) l.Fa[m] = *p++;
    for (int m = 0; m < MM; ++m) l.Far[m] = *p++;
    l.Fru[0] = *p++;
    l.Fru[1] = *p++;
    l.FE = *p++;
    l.Ss = *p++;
    FS a, b;
    zero(a);
    zero(b);
    hllc_rev(M, *(const FS*)L, *(const FS*)R, d, l, a, b);
    *(FS*)lL = a;
    *(FS*)lR = b;
}

void h_c2p(int M, const double* e, const double* c, double* out)
{
    Carried o;
    zero(o);
    c2p_fwd(eos_of(M, e), *(const Cons*)c, o);
    *(Carried*)out = o;
}

void h_c2p_rev(int M, const double* e, const double* c, const double* lam, double* mu, double* ge)
{
    GradEos g;
    zero(g);
    Cons r;
    zero(r);
    c2p_rev(eos_of(M, e), *(const Cons*)c, *(const Carried*)lam, r, g);
    *(Cons*)mu = r;
    put_grad(g, ge);
}

void h_p2c(int M, const double* e, const double* x, double* out)
{
    Carried o;
    zero(o);
    p2c_state_fwd(eos_of(M, e), *(const Prim*)x, o);
    *(Carried*)out = o;
}

void h_p2c_rev(int M, const double* e, const double* x, const double* lam, double* lx, double* ge)
{
    GradEos g;
    zero(g);
    Prim r;
    zero(r);
    p2c_state_rev(eos_of(M, e), *(const Prim*)x, *(const Carried*)lam, r, g);
    *(Prim*)lx = r;
    put_grad(g, ge);
}

int h_thinc(const double* s, int d, double beta0, double dx, double dy, double* LR)
{
    double S[3][3];
    for (int i = 0; i < 9; ++i) S[i / 3][i % 3] = s[i];
    return thinc_cand_fwd(S, d, beta0, dx, dy, ch, th, ex, LR[0], LR[1]) ? 1 : 0;
}

void h_thinc_rev(const double* s, int d, double beta0, double dx, double dy, double lL, double lR, double* ls)
{
    double S[3][3], LS[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int i = 0; i < 9; ++i) S[i / 3][i % 3] = s[i];
    thinc_cand_rev(S, d, beta0, dx, dy, ch, th, ex, lL, lR, LS);
    for (int i = 0; i < 9; ++i) ls[i] = LS[i / 3][i % 3];
}

// the MUSCL extrapolation of one variable (hllc.cpp:527-568)
void h_muscl(double um, double u0, double up, double* lr) { muscl_fwd(um, u0, up, lr[0], lr[1]); }

void h_muscl_rev(double um, double u0, double up, double lul, double lur, double* out)
{
    muscl_rev(muscl_branch(um, u0, up), lul, lur, out[0], out[1], out[2]);
}
}
