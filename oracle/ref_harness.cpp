// Oracle harness: drives the reference's own hot-path sources (compiled
// unchanged from the reference tree against oracle/amrex_lite and
// oracle/shims) through the per-timestep update. TEST INFRASTRUCTURE ONLY.
//
// It replaces the two reference files that need libconfig++ / ParmParse
// (main.cpp, initialise.cpp) with:
//   * an input file (written by tenjin_gb300-independent Python in tests/)
//     holding the parameters and the initial primitive state;
//   * setInitialConditions' last step, BoxAccessCellArray::
//     primitiveToConservative per box (initialise.cpp:111-123);
//   * the time loop restated from main.cpp:121-191 (halo fill, getTimeStep,
//     clamp to finalT, dt*=0.2 for n<5, U=U1, advance, plasticUpdate,
//     cleanUpV, cleanUpAlpha, NaN stop), with a step cap.
// Several independent domains may be given; they share one dt, the minimum
// of their getTimeStep results (the batched-box workload).
// The copper Hugoniot Mie-Gruneisen EOS has no reference implementation; it
// is defined here with the reference's EOS interface (equationofstate.h).
//
// Usage: tenjin_ref_<D>d <input.bin> <output.bin>
#include "simulationheader.h"
#include "timestep.h"

#include <cstdint>
#include <cstring>
#include <fstream>

// Linear us-up Hugoniot reference curve with constant Gruneisen gamma:
// params = {adiabaticIndex(=Gamma0+1), pref, eref, CV, rho0, c0, s, G0}.
class HugoniotSolidEOS : public MieGruneisenEOS {
public:
    void define(Vector<Real>& p) override
    {
        adiabaticIndex = p[0];
        GruneisenGamma = adiabaticIndex - 1.0;
        pref = p[1];
        eref = p[2];
        CV = p[3];
        rho0 = p[4];
        c0 = p[5];
        s = p[6];
        G0 = p[7];
    }
    Real eta(BoxAccessCellArray& U, int i, int j, int k, int m) { return 1.0 - rho0 / U(i, j, k, RHO_K, m); }
    Real pH(Real e) { Real d = 1.0 - s * e; return rho0 * c0 * c0 * e / (d * d); }
    Real dpHdeta(Real e) { Real d = 1.0 - s * e; return rho0 * c0 * c0 * (1.0 + s * e) / (d * d * d); }
    Real coldCompressionInternalEnergy(BoxAccessCellArray& U, int i, int j, int k, int m) override
    {
        Real e = eta(U, i, j, k, m);
        return U(i, j, k, ALPHARHO, m) * (pH(e) * e / (2.0 * rho0));
    }
    Real coldCompressionPressure(BoxAccessCellArray& U, int i, int j, int k, int m) override
    {
        Real e = eta(U, i, j, k, m);
        return (U(i, j, k, ALPHA, m) / GruneisenGamma) * pH(e);
    }
    Real getSoundSpeedContribution(BoxAccessCellArray& U, int i, int j, int k, int m) override
    {
        Real rho = U(i, j, k, RHO_K, m);
        Real e = eta(U, i, j, k, m);
        Real detadrho = rho0 / (rho * rho);
        Real dp = dpHdeta(e) * detadrho;
        Real de = (pH(e) + e * dpHdeta(e)) / (2.0 * rho0) * detadrho;
        return dp - GruneisenGamma * rho * de + (U(i, j, k, P) * (GruneisenGamma + 1.0) - pH(e)) / rho +
               (4.0 / 3.0) * G0 / rho;
    }
    Real componentShearModulus(BoxAccessCellArray&, int, int, int, int) override { return G0; }
    Real dGdrho(BoxAccessCellArray&, int, int, int, int) override { return 0.0; }
    Real dG2drho2(BoxAccessCellArray&, int, int, int, int) override { return 0.0; }
    Real transverseWaveSpeedContribution(BoxAccessCellArray& U, int i, int j, int k, int m) override
    {
        return U(i, j, k, ALPHA, m) * G0 / (U(i, j, k, RHO_K, m) * GruneisenGamma);
    }
    Real shearInternalEnergy(BoxAccessCellArray& U, int i, int j, int k, int m) override
    {
        return U(i, j, k, ALPHA, m) * (G0 * U(i, j, k, HJ2));
    }
    Real shearPressure(BoxAccessCellArray& U, int i, int j, int k, int m) override
    {
        return (U(i, j, k, ALPHA, m) / GruneisenGamma) * ((U(i, j, k, RHO_K, m) * 0.0 - G0) * U(i, j, k, HJ2));
    }
    Real inverseGruneisen(BoxAccessCellArray& U, int i, int j, int k, int m) override
    {
        return U(i, j, k, ALPHA, m) / GruneisenGamma;
    }
    Real rho0, c0, s, G0;
};

namespace {

struct Reader {
    std::ifstream f;
    explicit Reader(const char* path) : f(path, std::ios::binary)
    {
        if (!f) { std::fprintf(stderr, "cannot open %s\n", path); std::exit(2); }
    }
    int32_t i32() { int32_t v; f.read((char*)&v, 4); return v; }
    // optional trailing word: `dflt` when the file ends first
    int32_t i32_or(int32_t dflt) { int32_t v; return f.read((char*)&v, 4) ? v : dflt; }
    double f64() { double v; f.read((char*)&v, 8); return v; }
    void arr(double* p, size_t n) { f.read((char*)p, 8 * n); }
};

struct Domain {
    int n_cells[3];
    double dimL[3];
    std::vector<Box> boxes;
    std::vector<std::vector<double>> prim;  // by field
};

struct Sim {
    ParameterStruct parameters;
    AccessPattern* ap = nullptr;
    BoxArray ba;
    DistributionMapping dm;
    Geometry geom;
    CellArray *U, *U1, *U2, *UL, *UR, *ULStar, *URStar, *UStarStar, *MUSCLgrad;
    THINCArray* THINCArr;
    TimeStep* timeStep;
    Array<MultiFab, AMREX_SPACEDIM> flux_arr;
    Vector<BCRec> bc;
};

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 3) { std::fprintf(stderr, "usage: %s in.bin out.bin [gnuplot-dir]\n", argv[0]); return 2; }

    Reader rd(argv[1]);
    if (rd.i32() != 0x544a4f52) { std::fprintf(stderr, "bad magic\n"); return 2; }
    int dim = rd.i32();
    if (dim != AMREX_SPACEDIM) { std::fprintf(stderr, "dim %d != build %d\n", dim, AMREX_SPACEDIM); return 2; }
    int M = rd.i32(), SOLID = rd.i32(), THINC = rd.i32(), PLASTIC = rd.i32(), MUSCL = rd.i32(), nghost = rd.i32();
    int lobc[3], hibc[3];
    for (int d = 0; d < 3; ++d) lobc[d] = rd.i32();
    for (int d = 0; d < 3; ++d) hibc[d] = rd.i32();
    double CFL = rd.f64(), beta = rd.f64(), finalT = rd.f64();
    int maxsteps = rd.i32();

    std::vector<int> phase(M), eostype(M);
    std::vector<Vector<Real>> eosparams(M);
    std::vector<double> yield(M);
    for (int m = 0; m < M; ++m) {
        phase[m] = rd.i32();
        eostype[m] = rd.i32();
        int np = rd.i32();
        eosparams[m].resize(np);
        for (int q = 0; q < np; ++q) eosparams[m][q] = rd.f64();
        yield[m] = rd.f64();
    }
    int ndom = rd.i32();
    int nprim = M + M + 3 + 1 + (SOLID ? 9 : 0) + (PLASTIC ? M : 0);
    std::vector<Domain> doms(ndom);
    for (auto& D : doms) {
        for (int d = 0; d < 3; ++d) D.n_cells[d] = rd.i32();
        for (int d = 0; d < 3; ++d) D.dimL[d] = rd.f64();
        int nbox = rd.i32();
        for (int b = 0; b < nbox; ++b) {
            int lo[3], hi[3];
            for (int d = 0; d < 3; ++d) lo[d] = rd.i32();
            for (int d = 0; d < 3; ++d) hi[d] = rd.i32();
            D.boxes.push_back(Box(IntVect(lo[0], lo[1], lo[2]), IntVect(hi[0], hi[1], hi[2])));
        }
        long nc = (long)D.n_cells[0] * D.n_cells[1] * D.n_cells[2];
        D.prim.assign(nprim, std::vector<double>(nc));
        for (int q = 0; q < nprim; ++q) rd.arr(D.prim[q].data(), nc);
    }
    // trailer: RADIAL, REACTIVE, numberOfMixtures, the mixture flag of each
    // material, then the initial lambda of each domain (absent: all zero)
    const int RADIAL = rd.i32_or(0);
    const int REACTIVE = rd.i32_or(0);
    const int NMIX = rd.i32_or(0);
    std::vector<int> mixflag(M, 0);
    for (int m = 0; m < M; ++m) mixflag[m] = rd.i32_or(0);
    for (auto& D : doms) {
        long nc = (long)D.n_cells[0] * D.n_cells[1] * D.n_cells[2];
        for (int q = 0; q < NMIX; ++q) {
            D.prim.emplace_back(nc);
            rd.arr(D.prim.back().data(), nc);
        }
    }

    PlasticEOS plastic;
    plastic.yieldStress.assign(M, 0.0);

    std::vector<Sim> sims(ndom);
    std::vector<MieGruneisenEOS*> eos(M);
    for (int m = 0; m < M; ++m) {
        switch (eostype[m]) {
            case 0: eos[m] = new MieGruneisenEOS(); break;
            case 1: eos[m] = new RomenskiiSolidEOS(); break;
            case 2: eos[m] = new WilkinsSolidEOS(); break;
            case 3: eos[m] = new HugoniotSolidEOS(); break;
            case 4: eos[m] = new MixtureEOS(); break;
            default: std::fprintf(stderr, "bad eos\n"); return 2;
        }
        eos[m]->define(eosparams[m]);
        if (PLASTIC && phase[m] == 0) plastic.yieldStress[m] = yield[m];
    }

    for (int di = 0; di < ndom; ++di) {
        Sim& S = sims[di];
        Domain& D = doms[di];
        ParameterStruct& Prm = S.parameters;
        Prm.SOLID = SOLID; Prm.THINC = THINC; Prm.RADIAL = RADIAL; Prm.PLASTIC = PLASTIC; Prm.REACTIVE = REACTIVE; Prm.MUSCL = MUSCL;
        Prm.numberOfMaterials = M; Prm.numberOfMixtures = NMIX; Prm.Nghost = nghost; Prm.CFL = CFL; Prm.THINCbeta = beta;
        Prm.max_grid_size = 0; Prm.dt = 0.0; Prm.x0 = 0.0;
        for (int d = 0; d < AMREX_SPACEDIM; ++d) { Prm.n_cells[d] = D.n_cells[d]; Prm.dimL[d] = D.dimL[d]; }
        Prm.materialInfo.resize(M);
        for (int m = 0; m < M; ++m) {
            Prm.materialInfo[m].phase = phase[m] == 0 ? solid : fluid;
            Prm.materialInfo[m].mixture = mixflag[m];
            Prm.materialInfo[m].mixtureIndex = 0;  // getMaterialParameters (initialise.cpp:187)
            Prm.materialInfo[m].plastic = (PLASTIC && phase[m] == 0);
            Prm.materialInfo[m].EOS = eos[m];
        }
        IntVect lo(0, 0, 0), hi(D.n_cells[0] - 1, D.n_cells[1] - 1, D.n_cells[2] - 1);
        Box domain(lo, hi);
        S.ba.boxes = D.boxes;
        S.geom = Geometry(domain, RealBox({AMREX_D_DECL(0.0, 0.0, 0.0)}, {AMREX_D_DECL(D.dimL[0], D.dimL[1], D.dimL[2])}),
                          CoordSys::cartesian, {AMREX_D_DECL(0, 0, 0)});
        Prm.dx = {S.geom.CellSize()[0], S.geom.CellSize()[1], S.geom.CellSize()[2]};
        S.ap = new AccessPattern(Prm);
        Prm.Ncomp = S.ap->variableNames.size();
        int Nc = Prm.Ncomp;
        S.U = new CellArray(S.ba, S.dm, Nc, nghost, *S.ap, Prm);
        S.U1 = new CellArray(S.ba, S.dm, Nc, nghost, *S.ap, Prm);
        S.U2 = new CellArray(S.ba, S.dm, Nc, nghost, *S.ap, Prm);
        S.UL = new CellArray(S.ba, S.dm, Nc, nghost, *S.ap, Prm);
        S.UR = new CellArray(S.ba, S.dm, Nc, nghost, *S.ap, Prm);
        S.ULStar = new CellArray(S.ba, S.dm, Nc, nghost, *S.ap, Prm);
        S.URStar = new CellArray(S.ba, S.dm, Nc, nghost, *S.ap, Prm);
        S.UStarStar = new CellArray(S.ba, S.dm, Nc, nghost, *S.ap, Prm);
        S.MUSCLgrad = new CellArray(S.ba, S.dm, Nc, nghost, *S.ap, Prm);
        S.THINCArr = new THINCArray(S.ba, S.dm, nghost, Prm);
        S.timeStep = new TimeStep(S.ba, S.dm, AMREX_SPACEDIM, nghost);
        for (int dir = 0; dir < AMREX_SPACEDIM; ++dir) {
            BoxArray edge_ba = S.ba;
            edge_ba.surroundingNodes(dir);
            S.flux_arr[dir].define(edge_ba, S.dm, Nc, 0);
        }
        S.bc.assign(Nc, BCRec());
        InitialStruct initial;
        for (int d = 0; d < AMREX_SPACEDIM; ++d) { initial.lowBoundary[d] = lobc[d]; initial.highBoundary[d] = hibc[d]; }
        setBoundaryConditions(S.bc, Prm, initial, *S.ap);

        // Initial state: primitive fields, then primitiveToConservative per box
        // (initialise.cpp:111-123).
        for (MFIter mfi(S.U1->data); mfi.isValid(); ++mfi) {
            const Box& bx = mfi.validbox();
            BoxAccessCellArray U(mfi, bx, *S.U1);
            for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
                for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
                    for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) {
                        long c = i + (long)D.n_cells[0] * (j + (long)D.n_cells[1] * k);
                        int q = 0;
                        for (int m = 0; m < M; ++m) U(i, j, k, ALPHA, m) = D.prim[q++][c];
                        for (int m = 0; m < M; ++m) U(i, j, k, RHO_K, m) = D.prim[q++][c];
                        for (int r = 0; r < 3; ++r) U(i, j, k, VELOCITY, 0, r) = D.prim[q++][c];
                        U(i, j, k, P) = D.prim[q++][c];
                        if (SOLID)
                            for (int r = 0; r < 3; ++r)
                                for (int cc = 0; cc < 3; ++cc) U(i, j, k, V_TENSOR, 0, r, cc) = D.prim[q++][c];
                        if (PLASTIC)
                            for (int m = 0; m < M; ++m) U(i, j, k, EPSILON, m) = D.prim[q++][c];
                        for (int m = 0; m < M; ++m)  // initialise.cpp:66-71
                            if (mixflag[m]) {
                                U(i, j, k, RHO_MIX, m, 0) = U(i, j, k, RHO_K, m);
                                U(i, j, k, RHO_MIX, m, 1) = U(i, j, k, RHO_K, m);
                                U(i, j, k, LAMBDA, m) = D.prim[q++][c];
                            }
                    }
            U.primitiveToConservative();
        }
    }

    // Time loop restated from main.cpp:121-191.
    std::vector<double> dts;
    double t = 0.0;
    int n = 0;
    double t0 = amrex::second();
    bool nan_stop = false;
    double dt = 0.0;
    for (; t < finalT && n < maxsteps; t += dt, n++) {
        dt = std::numeric_limits<double>::max();
        for (auto& S : sims) {
            FillDomainBoundary(S.U1->data, S.geom, S.bc);
            S.U1->data.FillBoundary(S.geom.periodicity());
            double d = S.timeStep->getTimeStep(*S.U1, S.parameters);
            dt = (d < dt ? d : dt);
        }
        if (t + dt > finalT) dt = finalT - t;
        if (n < 5) dt *= 0.2;
        for (auto& S : sims) {
            ParameterStruct& Prm = S.parameters;
            Prm.dt = dt;
            *S.U = *S.U1;
            advance(*S.U, *S.U1, *S.U2, *S.UL, *S.UR, *S.MUSCLgrad, *S.ULStar, *S.URStar, *S.UStarStar, S.flux_arr,
                    S.geom, Prm, S.bc, *S.THINCArr);
            if (Prm.REACTIVE) reactiveUpdate(*S.U, *S.U1, *S.U2, Prm);
            if (Prm.PLASTIC) plastic.plasticUpdate(*S.U1, Prm);
            if (Prm.RADIAL) geometricSourceTerm(*S.U1, Prm);
            if (Prm.SOLID) S.U1->cleanUpV();
            S.U1->cleanUpAlpha();
            if (S.U1->contains_nan()) nan_stop = true;
        }
        dts.push_back(dt);
        if (nan_stop) break;
    }
    double elapsed = amrex::second() - t0;
    // optional: the reference's 1-D gnuplot dump of the final state of the
    // first domain (print.cpp:33-43), picture 0, into the directory argv[3]
    if (argc > 3) PrintAllVarsTo1DGnuplotFile(*sims[0].U1, 0, std::string(argv[3]));

    std::ofstream out(argv[2], std::ios::binary);
    int32_t hdr[4] = {0x544a4f55, (int32_t)dts.size(), nan_stop ? 1 : 0, sims[0].parameters.Ncomp};
    out.write((char*)hdr, sizeof hdr);
    out.write((char*)&t, 8);
    out.write((char*)&elapsed, 8);
    out.write((char*)dts.data(), 8 * dts.size());
    for (int di = 0; di < ndom; ++di) {
        Sim& S = sims[di];
        Domain& D = doms[di];
        long nc = (long)D.n_cells[0] * D.n_cells[1] * D.n_cells[2];
        int Nc = S.parameters.Ncomp;
        std::vector<double> buf((size_t)nc * Nc);
        for (MFIter mfi(S.U1->data); mfi.isValid(); ++mfi) {
            const Box& bx = mfi.validbox();
            auto a = S.U1->data[mfi].array();
            for (int q = 0; q < Nc; ++q)
                for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
                    for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
                        for (int i = bx.lo[0]; i <= bx.hi[0]; ++i)
                            buf[(size_t)q * nc + i + (long)D.n_cells[0] * (j + (long)D.n_cells[1] * k)] = a(i, j, k, q);
        }
        out.write((char*)buf.data(), 8 * buf.size());
    }
    return 0;
}
