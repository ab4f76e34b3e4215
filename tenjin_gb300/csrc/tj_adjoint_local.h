// Reverse-mode (adjoint) derivatives of the local operators of the 2-D fluid
// update, one cell or one face at a time. Each *_rev function takes the
// forward inputs, recomputes the forward intermediates it needs and maps the
// adjoint of the outputs to the adjoint of the inputs; adjoints of the EOS
// parameters are added into a GradEos. Discrete choices (limiter branch, wave
// ordering, clamps) are taken at their forward values: the derivative is that
// of the active branch.
//
// Operators and the reference code they differentiate:
//   cleanup_rev      cleanUpAlpha (boxaccesscellarray.cpp:530-599)
//   face_state_rev   cleanUpAlpha of a reconstructed state, then
//                    primitiveToConservative (:124-174) and getSoundSpeed
//                    (:254-285) (hllc.cpp:628-638)
//   hllc_rev         calc_fluxes / getSstar / getStarState (hllc.cpp:5-73,384-487)
//   c2p_rev          conservativeToPrimitive (boxaccesscellarray.cpp:67-122)
//   p2c_state_rev    primitiveToConservative of the initial state (initialise.cpp:111-123)
//   thinc_cand_rev   THINC candidate values of one material (thinc.cpp:28-147)
//   muscl_branch     the active branch of the van Leer MUSCL slope (hllc.cpp:527-568)
// The equation of state is the stiffened-gas Mie-Gruneisen form
// (equationofstate.cpp:37-64): e_cold = e_ref alpha rho, p_cold = p_ref alpha / G,
// c^2 = (p (G + 1) - p_ref) / rho_k, xi = 1 / G, with G = params[0] - 1.
//
// The header is plain C++ so that it also compiles for the host, where the
// local derivatives are checked against finite differences.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define TJA_HD __host__ __device__ inline
#define TJA_NOTFINITE(x) (isinf(x) || isnan(x))
#else
#define TJA_HD inline
#define TJA_NOTFINITE(x) (std::isinf(x) || std::isnan(x))
#endif

namespace tja {

constexpr int MM = 4;  // materials

struct Eos {
    int M;
    double G[MM], pr[MM], er[MM];  // G = params[0] - 1, p_ref = params[1], e_ref = params[2]
};

struct GradEos {
    double G[MM], pr[MM], er[MM];
};

// reconstructed primitive values of one side of a cell (alpha before cleanUpAlpha)
struct Prim {
    double a[MM], rk[MM], u[2], p;
};

// a face state after cleanUpAlpha, primitiveToConservative and getSoundSpeed
struct FS {
    double a[MM], ar[MM], rho, ru[2], u[2], E, p, c;
};

// conserved words of a cell: alpha, alpha rho, rho u, E
struct Cons {
    double a[MM], ar[MM], ru[2], E;
};

// the carried words of a cell (2-D fluids)
struct Carried {
    double a[MM], ar[MM], rk[MM], rho, ru[2], u[2], E, p;
};

TJA_HD void zero(GradEos& g)
{
    for (int m = 0; m < MM; ++m) g.G[m] = g.pr[m] = g.er[m] = 0.0;
}
TJA_HD void zero(Prim& x)
{
    for (int m = 0; m < MM; ++m) x.a[m] = x.rk[m] = 0.0;
    x.u[0] = x.u[1] = x.p = 0.0;
}
TJA_HD void zero(FS& x)
{
    for (int m = 0; m < MM; ++m) x.a[m] = x.ar[m] = 0.0;
    x.rho = x.ru[0] = x.ru[1] = x.u[0] = x.u[1] = x.E = x.p = x.c = 0.0;
}
TJA_HD void zero(Cons& x)
{
    for (int m = 0; m < MM; ++m) x.a[m] = x.ar[m] = 0.0;
    x.ru[0] = x.ru[1] = x.E = 0.0;
}
TJA_HD void zero(Carried& x)
{
    for (int m = 0; m < MM; ++m) x.a[m] = x.ar[m] = x.rk[m] = 0.0;
    x.rho = x.ru[0] = x.ru[1] = x.u[0] = x.u[1] = x.E = x.p = 0.0;
}

// ---------------------------------------------------------------------------
// cleanUpAlpha: clamp (< 0 -> 1e-6, > 1 -> 1) and renormalise to sum 1.
// ---------------------------------------------------------------------------
TJA_HD void cleanup_fwd(int M, const double* a, double* out)
{
    double tot = 0.0, c[MM];
    for (int m = 0; m < M; ++m) {
        double v = a[m];
        if (v < 0.0) v = 1E-6;
        else if (v > 1.0) v = 1.0;
        c[m] = v;
        tot += v;
    }
    for (int m = 0; m < M; ++m) out[m] = c[m] * (1.0 / tot);
}

// lam_in = (d cleanup / d a)^T lam_out
TJA_HD void cleanup_rev(int M, const double* a, const double* lam_out, double* lam_in)
{
    double tot = 0.0, c[MM];
    for (int m = 0; m < M; ++m) {
        double v = a[m];
        if (v < 0.0) v = 1E-6;
        else if (v > 1.0) v = 1.0;
        c[m] = v;
        tot += v;
    }
    double s = 0.0;
    for (int m = 0; m < M; ++m) s += lam_out[m] * c[m];
    const double it = 1.0 / tot;
    for (int m = 0; m < M; ++m) {
        const bool in = !(a[m] < 0.0) && !(a[m] > 1.0);
        lam_in[m] = in ? (lam_out[m] * it - s * it * it) : 0.0;
    }
}

// ---------------------------------------------------------------------------
// Face state: [cleanUpAlpha], primitiveToConservative, getSoundSpeed.
// ---------------------------------------------------------------------------
TJA_HD void face_state_fwd(const Eos& E, const Prim& x, bool clean, FS& s)
{
    const int M = E.M;
    if (clean) cleanup_fwd(M, x.a, s.a);
    else
        for (int m = 0; m < M; ++m) s.a[m] = x.a[m];
    s.rho = 0.0;
    for (int m = 0; m < M; ++m) {
        s.ar[m] = s.a[m] * x.rk[m];
        s.rho += s.ar[m];
    }
    double ke = 0.0;
    for (int r = 0; r < 2; ++r) {
        s.u[r] = x.u[r];
        s.ru[r] = x.u[r] * s.rho;
        ke += 0.5 * s.rho * x.u[r] * x.u[r];
    }
    s.p = x.p;
    double invG = 0.0, ent = 0.0, pnt = 0.0;
    for (int m = 0; m < M; ++m) {
        invG += s.a[m] / E.G[m];
        ent += E.er[m] * s.ar[m];
        pnt += E.pr[m] * s.a[m] / E.G[m];
    }
    s.E = x.p * invG + ent - pnt + ke;
    double A = 0.0, xit = 0.0;
    for (int m = 0; m < M; ++m) {
        const double xi = 1.0 / E.G[m];
        const double c2 = x.p * (E.G[m] + 1.0) / x.rk[m] - E.pr[m] / x.rk[m];
        const double v = xi * c2 * s.ar[m] / s.rho;
        A += (0.0 < v) ? v : 0.0;
        xit += xi * s.a[m];
    }
    if (A <= 0.0) A = 1E-6;
    s.c = sqrt(A / xit);
}

TJA_HD void face_state_rev(const Eos& E, const Prim& x, bool clean, const FS& l, Prim& lx, GradEos& g)
{
    const int M = E.M;
    FS s;
    face_state_fwd(E, x, clean, s);
    double la[MM], lar[MM], lrk[MM];
    for (int m = 0; m < M; ++m) {
        la[m] = l.a[m];
        lar[m] = l.ar[m];
        lrk[m] = 0.0;
    }
    double lrho = l.rho, lp = l.p, lu[2] = {l.u[0], l.u[1]};
    // getSoundSpeed: c = sqrt(A / xit)
    {
        double A = 0.0, xit = 0.0;
        for (int m = 0; m < M; ++m) {
            const double xi = 1.0 / E.G[m];
            const double c2 = x.p * (E.G[m] + 1.0) / x.rk[m] - E.pr[m] / x.rk[m];
            const double v = xi * c2 * s.ar[m] / s.rho;
            A += (0.0 < v) ? v : 0.0;
            xit += xi * s.a[m];
        }
        const bool floored = A <= 0.0;
        const double lA = floored ? 0.0 : l.c / (2.0 * s.c * xit);
        const double lxit = -l.c * s.c / (2.0 * xit);
        for (int m = 0; m < M; ++m) {
            const double xi = 1.0 / E.G[m];
            const double c2 = x.p * (E.G[m] + 1.0) / x.rk[m] - E.pr[m] / x.rk[m];
            const double v = xi * c2 * s.ar[m] / s.rho;
            double lxi = lxit * s.a[m];
            la[m] += lxit * xi;
            if (0.0 < v) {
                const double lc2 = lA * xi * s.ar[m] / s.rho;
                lar[m] += lA * xi * c2 / s.rho;
                lrho += -lA * v / s.rho;
                lxi += lA * c2 * s.ar[m] / s.rho;
                lp += lc2 * (E.G[m] + 1.0) / x.rk[m];
                lrk[m] += -lc2 * c2 / x.rk[m];
                g.G[m] += lc2 * x.p / x.rk[m];
                g.pr[m] += -lc2 / x.rk[m];
            }
            g.G[m] += -lxi * xi * xi;
        }
    }
    // primitiveToConservative: E = p invG + sum e_ref ar - sum p_ref a / G + ke
    {
        const double lE = l.E;
        double invG = 0.0;
        for (int m = 0; m < M; ++m) invG += s.a[m] / E.G[m];
        lp += lE * invG;
        for (int m = 0; m < M; ++m) {
            la[m] += lE * (x.p - E.pr[m]) / E.G[m];
            g.G[m] += -lE * (x.p - E.pr[m]) * s.a[m] / (E.G[m] * E.G[m]);
            g.pr[m] += -lE * s.a[m] / E.G[m];
            g.er[m] += lE * s.ar[m];
            lar[m] += lE * E.er[m];
        }
        for (int r = 0; r < 2; ++r) {
            lrho += lE * 0.5 * x.u[r] * x.u[r] + l.ru[r] * x.u[r];
            lu[r] += lE * s.rho * x.u[r] + l.ru[r] * s.rho;
        }
    }
    for (int m = 0; m < M; ++m) {
        lar[m] += lrho;
        la[m] += lar[m] * x.rk[m];
        lrk[m] += lar[m] * s.a[m];
    }
    if (clean) cleanup_rev(M, x.a, la, lx.a);
    else
        for (int m = 0; m < M; ++m) lx.a[m] = la[m];
    for (int m = 0; m < M; ++m) lx.rk[m] = lrk[m];
    lx.u[0] = lu[0];
    lx.u[1] = lu[1];
    lx.p = lp;
}

// ---------------------------------------------------------------------------
// HLLC flux of a face along d. F holds alpha[M], alphaRho[M], rhoU[2], E.
// ---------------------------------------------------------------------------
struct HllcOut {
    double Fa[MM], Far[MM], Fru[2], FE, Ss;
    int side;
};

TJA_HD void hllc_fwd(int M, const FS& L, const FS& R, int d, HllcOut& o)
{
    const double uL = L.u[d], uR = R.u[d];
    const double x1 = fabs(uL) + L.c, x2 = fabs(uR) + R.c;
    const double SR = (x1 < x2) ? x2 : x1;
    const double SL = -SR;
    const double Ss = (R.p - L.p + L.ru[d] * (SL - uL) - R.ru[d] * (SR - uR)) / (L.rho * (SL - uL) - R.rho * (SR - uR));
    o.Ss = Ss;
    int side;
    bool hllc;
    if (SL >= 0.0) { side = 0; hllc = false; }
    else if (Ss >= 0.0) { side = 0; hllc = true; }
    else if (SR >= 0.0) { side = 1; hllc = true; }
    else { side = 1; hllc = false; }
    o.side = side;
    const FS& K = side ? R : L;
    const double SK = side ? SR : SL, uK = K.u[d];
    const double mult = (fabs((Ss - uK) / Ss) < 1E-20) ? 1.0 : (SK - uK) / (SK - Ss);
    double ars[MM], rs = 0.0;
    for (int m = 0; m < M; ++m) {
        ars[m] = mult * K.ar[m];
        rs += ars[m];
    }
    double rus[2];
    rus[d] = mult * K.rho * Ss;
    rus[1 - d] = mult * K.ru[1 - d];
    const double vsd = rus[d] / rs;
    const double Es = mult * K.rho * (K.E / K.rho + (Ss - uK) * (Ss + K.p / (K.rho * (SK - uK))));
    const double w = hllc ? SK : 0.0;
    for (int m = 0; m < M; ++m) {
        o.Fa[m] = K.a[m] * vsd;
        o.Far[m] = K.ar[m] * uK + w * (ars[m] - K.ar[m]);
    }
    for (int r = 0; r < 2; ++r) o.Fru[r] = K.ru[r] * uK + (r == d ? K.p : 0.0) + w * (rus[r] - K.ru[r]);
    o.FE = (K.E + K.p) * uK + w * (Es - K.E);
}

// lF: adjoint of (Fa, Far, Fru, FE, Ss); lL, lR: adjoint of the face states
// (added to). Returns S*.
TJA_HD double hllc_rev(int M, const FS& L, const FS& R, int d, const HllcOut& lF, FS& lL, FS& lR)
{
    const double uL = L.u[d], uR = R.u[d];
    const double x1 = fabs(uL) + L.c, x2 = fabs(uR) + R.c;
    const double SR = (x1 < x2) ? x2 : x1;
    const double SL = -SR;
    const double Num = R.p - L.p + L.ru[d] * (SL - uL) - R.ru[d] * (SR - uR);
    const double Den = L.rho * (SL - uL) - R.rho * (SR - uR);
    const double Ss = Num / Den;
    int side;
    bool hllc;
    if (SL >= 0.0) { side = 0; hllc = false; }
    else if (Ss >= 0.0) { side = 0; hllc = true; }
    else if (SR >= 0.0) { side = 1; hllc = true; }
    else { side = 1; hllc = false; }
    const FS& K = side ? R : L;
    FS& lK = side ? lR : lL;
    const double SK = side ? SR : SL, uK = K.u[d];
    const bool guard = fabs((Ss - uK) / Ss) < 1E-20;
    const double mult = guard ? 1.0 : (SK - uK) / (SK - Ss);
    double ars[MM], rs = 0.0;
    for (int m = 0; m < M; ++m) {
        ars[m] = mult * K.ar[m];
        rs += ars[m];
    }
    double rus[2];
    rus[d] = mult * K.rho * Ss;
    rus[1 - d] = mult * K.ru[1 - d];
    const double vsd = rus[d] / rs;
    const double D1 = Ss - uK, D2 = K.rho * Ss + K.p / (SK - uK);
    const double W = K.E + D1 * D2;
    const double Es = mult * W;
    const double w = hllc ? SK : 0.0;

    double lSs = lF.Ss, lSK = 0.0, luK = 0.0, lmult = 0.0, lvsd = 0.0;
    double lars[MM], lrus[2] = {0.0, 0.0}, lEs = 0.0;
    // alpha flux: Fa = K.a vsd
    for (int m = 0; m < M; ++m) {
        lK.a[m] += lF.Fa[m] * vsd;
        lvsd += lF.Fa[m] * K.a[m];
    }
    // Far = K.ar uK + w (ars - K.ar)
    for (int m = 0; m < M; ++m) {
        lK.ar[m] += lF.Far[m] * (uK - w);
        luK += lF.Far[m] * K.ar[m];
        lars[m] = lF.Far[m] * w;
        if (hllc) lSK += lF.Far[m] * (ars[m] - K.ar[m]);
    }
    // Fru = K.ru uK + p delta + w (rus - K.ru)
    for (int r = 0; r < 2; ++r) {
        lK.ru[r] += lF.Fru[r] * (uK - w);
        luK += lF.Fru[r] * K.ru[r];
        if (r == d) lK.p += lF.Fru[r];
        lrus[r] = lF.Fru[r] * w;
        if (hllc) lSK += lF.Fru[r] * (rus[r] - K.ru[r]);
    }
    // FE = (K.E + K.p) uK + w (Es - K.E)
    lK.E += lF.FE * (uK - w);
    lK.p += lF.FE * uK;
    luK += lF.FE * (K.E + K.p);
    lEs = lF.FE * w;
    if (hllc) lSK += lF.FE * (Es - K.E);
    // vsd = rus_d / rs
    lrus[d] += lvsd / rs;
    const double lrs = -lvsd * vsd / rs;
    for (int m = 0; m < M; ++m) lars[m] += lrs;
    // ars = mult K.ar; rus_d = mult K.rho Ss; rus_o = mult K.ru_o
    for (int m = 0; m < M; ++m) {
        lmult += lars[m] * K.ar[m];
        lK.ar[m] += lars[m] * mult;
    }
    lmult += lrus[d] * K.rho * Ss;
    lK.rho += lrus[d] * mult * Ss;
    lSs += lrus[d] * mult * K.rho;
    lmult += lrus[1 - d] * K.ru[1 - d];
    lK.ru[1 - d] += lrus[1 - d] * mult;
    // Es = mult W, W = K.E + D1 D2
    lmult += lEs * W;
    const double lW = lEs * mult;
    lK.E += lW;
    const double lD1 = lW * D2, lD2 = lW * D1;
    lSs += lD1;
    luK -= lD1;
    lK.rho += lD2 * Ss;
    lSs += lD2 * K.rho;
    lK.p += lD2 / (SK - uK);
    lSK += -lD2 * K.p / ((SK - uK) * (SK - uK));
    luK += lD2 * K.p / ((SK - uK) * (SK - uK));
    // mult = (SK - uK) / (SK - Ss)
    if (!guard) {
        const double den = SK - Ss;
        lSK += lmult * (uK - Ss) / (den * den);
        luK += -lmult / den;
        lSs += lmult * mult / den;
    }
    double lSL = 0.0, lSR = 0.0;
    if (side) lSR += lSK;
    else lSL += lSK;
    lK.u[d] += luK;
    // Ss = Num / Den
    const double lNum = lSs / Den, lDen = -lSs * Ss / Den;
    lR.p += lNum;
    lL.p -= lNum;
    lL.ru[d] += lNum * (SL - uL);
    lSL += lNum * L.ru[d];
    lL.u[d] -= lNum * L.ru[d];
    lR.ru[d] -= lNum * (SR - uR);
    lSR -= lNum * R.ru[d];
    lR.u[d] += lNum * R.ru[d];
    lL.rho += lDen * (SL - uL);
    lSL += lDen * L.rho;
    lL.u[d] -= lDen * L.rho;
    lR.rho -= lDen * (SR - uR);
    lSR -= lDen * R.rho;
    lR.u[d] += lDen * R.rho;
    // SL = -SR; SR = max(|uL| + cL, |uR| + cR)
    lSR -= lSL;
    if (x1 < x2) {
        lR.u[d] += lSR * ((uR > 0.0) - (uR < 0.0));
        lR.c += lSR;
    } else {
        lL.u[d] += lSR * ((uL > 0.0) - (uL < 0.0));
        lL.c += lSR;
    }
    return Ss;
}

// ---------------------------------------------------------------------------
// conservativeToPrimitive of a stage output: from the conserved words, the
// carried words rho_k, rho, u, p. lam is the adjoint of all carried words;
// mu (out) the adjoint of the conserved words.
// ---------------------------------------------------------------------------
TJA_HD void c2p_fwd(const Eos& E, const Cons& c, Carried& o)
{
    const int M = E.M;
    o.rho = 0.0;
    for (int m = 0; m < M; ++m) {
        o.a[m] = c.a[m];
        o.ar[m] = c.ar[m];
        o.rk[m] = c.ar[m] / c.a[m];
        o.rho += c.ar[m];
    }
    double ke = 0.0;
    for (int r = 0; r < 2; ++r) {
        o.ru[r] = c.ru[r];
        o.u[r] = c.ru[r] / o.rho;
        ke += 0.5 * o.rho * o.u[r] * o.u[r];
    }
    o.E = c.E;
    double invG = 0.0, ent = 0.0, pnt = 0.0;
    for (int m = 0; m < M; ++m) {
        invG += c.a[m] / E.G[m];
        ent += E.er[m] * c.ar[m];
        pnt += E.pr[m] * c.a[m] / E.G[m];
    }
    o.p = (c.E - ke - ent + pnt) / invG;
}

TJA_HD void c2p_rev(const Eos& E, const Cons& c, const Carried& lam, Cons& mu, GradEos& g)
{
    const int M = E.M;
    Carried o;
    c2p_fwd(E, c, o);
    double D = 0.0;
    for (int m = 0; m < M; ++m) D += c.a[m] / E.G[m];
    const double lN = lam.p / D, lD = -lam.p * o.p / D;
    for (int m = 0; m < M; ++m) {
        mu.a[m] = lam.a[m] - lam.rk[m] * o.rk[m] / c.a[m] + lN * E.pr[m] / E.G[m] + lD / E.G[m];
        mu.ar[m] = lam.ar[m] + lam.rk[m] / c.a[m] - lN * E.er[m];
        g.G[m] += -(lN * E.pr[m] + lD) * c.a[m] / (E.G[m] * E.G[m]);
        g.pr[m] += lN * c.a[m] / E.G[m];
        g.er[m] += -lN * c.ar[m];
    }
    mu.E = lam.E + lN;
    double lrho = lam.rho;
    for (int r = 0; r < 2; ++r) {
        // ke = 0.5 rho u^2 with u = ru / rho
        const double lu = lam.u[r] - lN * o.rho * o.u[r];
        lrho += -lN * 0.5 * o.u[r] * o.u[r];
        mu.ru[r] = lam.ru[r] + lu / o.rho;
        lrho += -lu * o.u[r] / o.rho;
    }
    for (int m = 0; m < M; ++m) mu.ar[m] += lrho;
}

// ---------------------------------------------------------------------------
// primitiveToConservative of a full cell (the initial state): carried words
// from alpha, rho_k, u, p. lam: adjoint of the carried words; lx: adjoint of
// the primitives.
// ---------------------------------------------------------------------------
TJA_HD void p2c_state_fwd(const Eos& E, const Prim& x, Carried& o)
{
    const int M = E.M;
    o.rho = 0.0;
    for (int m = 0; m < M; ++m) {
        o.a[m] = x.a[m];
        o.rk[m] = x.rk[m];
        o.ar[m] = x.a[m] * x.rk[m];
        o.rho += o.ar[m];
    }
    double ke = 0.0;
    for (int r = 0; r < 2; ++r) {
        o.u[r] = x.u[r];
        o.ru[r] = x.u[r] * o.rho;
        ke += 0.5 * o.rho * x.u[r] * x.u[r];
    }
    o.p = x.p;
    double invG = 0.0, ent = 0.0, pnt = 0.0;
    for (int m = 0; m < M; ++m) {
        invG += x.a[m] / E.G[m];
        ent += E.er[m] * o.ar[m];
        pnt += E.pr[m] * x.a[m] / E.G[m];
    }
    o.E = x.p * invG + ent - pnt + ke;
}

TJA_HD void p2c_state_rev(const Eos& E, const Prim& x, const Carried& lam, Prim& lx, GradEos& g)
{
    const int M = E.M;
    Carried o;
    p2c_state_fwd(E, x, o);
    double invG = 0.0;
    for (int m = 0; m < M; ++m) invG += x.a[m] / E.G[m];
    const double lE = lam.E;
    double lar[MM];
    lx.p = lam.p + lE * invG;
    double lrho = lam.rho;
    for (int r = 0; r < 2; ++r) {
        lrho += lE * 0.5 * x.u[r] * x.u[r] + lam.ru[r] * x.u[r];
        lx.u[r] = lam.u[r] + lE * o.rho * x.u[r] + lam.ru[r] * o.rho;
    }
    for (int m = 0; m < M; ++m) {
        lar[m] = lam.ar[m] + lE * E.er[m] + lrho;
        lx.a[m] = lam.a[m] + lE * (x.p - E.pr[m]) / E.G[m] + lar[m] * x.rk[m];
        lx.rk[m] = lam.rk[m] + lar[m] * x.a[m];
        g.G[m] += -lE * (x.p - E.pr[m]) * x.a[m] / (E.G[m] * E.G[m]);
        g.pr[m] += -lE * x.a[m] / E.G[m];
        g.er[m] += lE * o.ar[m];
    }
}

// ---------------------------------------------------------------------------
// THINC candidate of one material at a cell, along d. s[di][dj] is alpha at
// (i + di - 1, j + dj - 1) (ghosts already mapped). Returns whether the cell
// is mixed; L and R are the candidate face values.
// ---------------------------------------------------------------------------
struct ThincMath {
    // transcendental functions used by the candidate (the caller's choice)
    double (*cosh_)(double);
    double (*tanh_)(double);
    double (*exp_)(double);
};

template <typename CoshF, typename TanhF, typename ExpF>
TJA_HD bool thinc_cand_fwd(const double s[3][3], int d, double beta0, double dx, double dy, CoshF ch, TanhF th, ExpF ex,
                           double& L, double& R)
{
    const double eps = 1E-20;
    const double aL = d == 0 ? s[0][1] : s[1][0], aR = d == 0 ? s[2][1] : s[1][2], a0 = s[1][1];
    const double mn = (aR < aL) ? aR : aL;
    const double mx = ((aL < aR) ? aR : aL) - mn;
    const double theta = (double)((0.0 < aR - aL) - (aR - aL < 0.0));
    const double C = (mx < eps) ? 0.0 : (a0 - mn + eps) / (mx + eps);
    const double delta = 1E-4;
    const bool mixed = (C > delta) && (C < (0.999999 - delta)) && ((aR - a0) * (a0 - aL) >= 0.0);
    L = R = 0.0;
    if (!mixed) return false;
    const double nx = -1.0 / (8.0 * dx) * (s[2][2] + 2.0 * s[2][1] + s[2][0] - s[0][2] - 2.0 * s[0][1] - s[0][0]);
    const double ny = -1.0 / (8.0 * dy) * (s[2][2] + 2.0 * s[1][2] + s[0][2] - s[0][0] - 2.0 * s[1][0] - s[2][0]);
    const double norm = sqrt(nx * nx + ny * ny);
    const double nvc = (norm < 1E-20) ? 0.0 : fabs((d == 0 ? nx : ny) / norm);
    const double beta = nvc * beta0 + 0.01;
    const double coshB = ch(beta), tanhB = th(beta);
    const double B = ex(theta * beta * ((2.0 * C) - 1.0));
    const double A = ((B / coshB) - 1.0) / tanhB;
    R = mn + (mx / 2.0) * (1.0 + theta * ((tanhB + A) / (1.0 + A * tanhB)));
    L = mn + (mx / 2.0) * (1.0 + theta * A);
    return true;
}

// ls[di][dj] += d(L, R)/ds^T (lL, lR); the cell must be mixed
template <typename CoshF, typename TanhF, typename ExpF>
TJA_HD void thinc_cand_rev(const double s[3][3], int d, double beta0, double dx, double dy, CoshF ch, TanhF th,
                           ExpF ex, double lL, double lR, double ls[3][3])
{
    const double eps = 1E-20;
    const double aL = d == 0 ? s[0][1] : s[1][0], aR = d == 0 ? s[2][1] : s[1][2], a0 = s[1][1];
    const double mn = (aR < aL) ? aR : aL;
    const double mx = ((aL < aR) ? aR : aL) - mn;
    const double theta = (double)((0.0 < aR - aL) - (aR - aL < 0.0));
    const double C = (a0 - mn + eps) / (mx + eps);
    const double nx = -1.0 / (8.0 * dx) * (s[2][2] + 2.0 * s[2][1] + s[2][0] - s[0][2] - 2.0 * s[0][1] - s[0][0]);
    const double ny = -1.0 / (8.0 * dy) * (s[2][2] + 2.0 * s[1][2] + s[0][2] - s[0][0] - 2.0 * s[1][0] - s[2][0]);
    const double norm = sqrt(nx * nx + ny * ny);
    const bool flat = norm < 1E-20;
    const double nd = d == 0 ? nx : ny;
    const double nvc = flat ? 0.0 : fabs(nd / norm);
    const double beta = nvc * beta0 + 0.01;
    const double coshB = ch(beta), tanhB = th(beta);
    const double B = ex(theta * beta * ((2.0 * C) - 1.0));
    const double A = ((B / coshB) - 1.0) / tanhB;
    const double q = 1.0 + A * tanhB;
    const double T = (tanhB + A) / q;

    double lmn = lL + lR;
    double lmx = lL * 0.5 * (1.0 + theta * A) + lR * 0.5 * (1.0 + theta * T);
    double lA = lL * (mx / 2.0) * theta;
    const double lT = lR * (mx / 2.0) * theta;
    double lt = lT * (1.0 - A * A) / (q * q);
    lA += lT * (1.0 - tanhB * tanhB) / (q * q);
    const double lB = lA / (coshB * tanhB);
    const double lch = -lA * B / (coshB * coshB * tanhB);
    lt += -lA * A / tanhB;
    double lbeta = lB * B * theta * (2.0 * C - 1.0);
    const double lC = lB * B * theta * beta * 2.0;
    lbeta += lch * tanhB * coshB;  // d cosh = sinh = tanh cosh
    lbeta += lt * (1.0 - tanhB * tanhB);
    const double lnvc = lbeta * beta0;
    // C = (a0 - mn + eps) / (mx + eps)
    double la0 = lC / (mx + eps);
    lmn -= lC / (mx + eps);
    lmx -= lC * C / (mx + eps);
    // mx = max - mn
    const double lmax = lmx;
    lmn -= lmx;
    double laL = 0.0, laR = 0.0;
    if (aR < aL) {
        laR += lmn;
        laL += lmax;
    } else {
        laL += lmn;
        laR += lmax;
    }
    if (d == 0) {
        ls[0][1] += laL;
        ls[2][1] += laR;
    } else {
        ls[1][0] += laL;
        ls[1][2] += laR;
    }
    ls[1][1] += la0;
    if (!flat) {
        const double sg = (double)((nd > 0.0) - (nd < 0.0));
        const double n3 = norm * norm * norm;
        const double lnx = lnvc * sg * ((d == 0 ? 1.0 : 0.0) / norm - nd * nx / n3);
        const double lny = lnvc * sg * ((d == 1 ? 1.0 : 0.0) / norm - nd * ny / n3);
        const double cx = -1.0 / (8.0 * dx) * lnx, cy = -1.0 / (8.0 * dy) * lny;
        ls[2][2] += cx + cy;
        ls[2][1] += 2.0 * cx;
        ls[2][0] += cx - cy;
        ls[0][2] += -cx + cy;
        ls[0][1] += -2.0 * cx;
        ls[0][0] += -cx - cy;
        ls[1][2] += 2.0 * cy;
        ls[1][0] += -2.0 * cy;
    }
}

// ---------------------------------------------------------------------------
// MUSCL slope (hllc.cpp:527-568): the slope equals u0 - um when 0 < r < 1,
// up - u0 when r >= 1, and 0 otherwise (r = (u0-um)/(up-u0), r <= 0, inf or
// NaN). Returns 1, 2 or 0 for those branches.
// ---------------------------------------------------------------------------
TJA_HD void muscl_fwd(double um, double u0, double up, double& l, double& r)
{
    double rr = (u0 - um) / (up - u0);
    if (TJA_NOTFINITE(rr)) rr = 0.0;
    double phi = 0.0;
    if (rr > 0.0) {
        const double a = 2.0 / (1.0 + rr), b = 2.0 * rr / (1.0 + rr);
        phi = (b < a) ? b : a;
    }
    const double grad = phi * 0.5 * (up - um);
    l = u0 - 0.5 * grad;
    r = u0 + 0.5 * grad;
}

TJA_HD int muscl_branch(double um, double u0, double up)
{
    double rr = (u0 - um) / (up - u0);
    if (TJA_NOTFINITE(rr)) rr = 0.0;
    if (rr <= 0.0) return 0;
    const double a = 2.0 / (1.0 + rr), b = 2.0 * rr / (1.0 + rr);
    return (b < a) ? 1 : 2;
}

// d(ul, ur) of one variable: adjoints of um, u0, up from those of ul, ur.
TJA_HD void muscl_rev(int branch, double lul, double lur, double& lum, double& lu0, double& lup)
{
    const double lg = 0.5 * (lur - lul);
    lum = 0.0;
    lu0 = lul + lur;
    lup = 0.0;
    if (branch == 1) {
        lum = -lg;
        lu0 += lg;
    } else if (branch == 2) {
        lu0 -= lg;
        lup = lg;
    }
}

}  // namespace tja
