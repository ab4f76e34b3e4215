// C ABI of libtenjin_gpu.so (include/tenjin_gpu.h): context management,
// domain/box bookkeeping, state exchange in the reference's FArrayBox layout
// and the time-loop operators, dispatched to the FP64 reference-faithful
// kernels or to the mixed-precision fused kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tj_fp64.cuh"
#include "tj_adjoint.cuh"
#include "tj_tangent.cuh"
#include "tj_adjoint_gen.cuh"
#include "tj_mixed.cuh"
#include "tj_layout.h"
#include "tj_types.h"

using namespace tj;

namespace {

// CUDA-event timing of every kernel launch. Pairs recorded while a graph is
// captured belong to that graph and are read after each of its launches;
// pairs recorded by direct launches are read at the next synchronisation.
struct EventProf : Prof {
    struct Pair {
        std::string name;
        cudaEvent_t a, b;
    };
    std::vector<Pair> pool;
    size_t cursor = 0, graph_end = 0;
    bool capturing = false;
    std::vector<std::pair<std::string, double>> totals;
    std::vector<std::pair<std::string, long long>> counts;

    void reserve(size_t n)
    {
        while (pool.size() < n) {
            Pair p;
            cudaEventCreate(&p.a);
            cudaEventCreate(&p.b);
            pool.push_back(p);
        }
    }
    void begin(const char* kernel, void* st) override
    {
        if (cursor >= pool.size()) {
            if (capturing) return;  // pool is sized before capture
            reserve(pool.size() + 256);
        }
        pool[cursor].name = kernel;
        record(pool[cursor].a, st);
    }
    void end(const char* kernel, void* st) override
    {
        (void)kernel;
        if (cursor >= pool.size()) return;
        record(pool[cursor].b, st);
        ++cursor;
    }
    // Inside a stream capture an event must be recorded as an external event
    // node to be recorded again each time the graph runs.
    void record(cudaEvent_t e, void* st)
    {
        if (capturing) cudaEventRecordWithFlags(e, (cudaStream_t)st, cudaEventRecordExternal);
        else cudaEventRecord(e, (cudaStream_t)st);
    }
    void add(const std::string& n, double ms)
    {
        for (auto& t : totals)
            if (t.first == n) { t.second += ms; for (auto& c : counts) if (c.first == n) c.second += 1; return; }
        totals.push_back({n, ms});
        counts.push_back({n, 1});
    }
    // Accumulate pairs [lo, hi) (the stream has been synchronised).
    void collect(size_t lo, size_t hi)
    {
        for (size_t i = lo; i < hi && i < pool.size(); ++i) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, pool[i].a, pool[i].b) == cudaSuccess) add(pool[i].name, ms);
            else cudaGetLastError();  // a pair that was not recorded: skip it
        }
    }
    void collect_direct()
    {
        collect(graph_end, cursor);
        cursor = graph_end;
    }
    ~EventProf() override
    {
        for (auto& p : pool) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    }
};

}  // namespace

struct tj_ctx {
    tj_params params;
    DevParams P;
    std::string err;
    cudaStream_t stream = nullptr;
    // geometry
    std::vector<DevDomain> doms;
    std::vector<std::vector<int>> boxes;  // per domain, 6 ints per box
    long long ntot = 0, nftot[3] = {0, 0, 0};
    bool geometry_dirty = true;  // box table not yet on the device
    // which copy of the state is current: the FP64 carried state A and/or the
    // fused kernels' state (precisions MIXED / FUSED64); conversions are made
    // when the other copy is next needed, not per call
    bool a_current = true, x_current = true;
    bool stage0_done = false;  // tj_advance_stage(0) saved U^n in C for stage 1
    // device memory
    DevDomain* d_doms = nullptr;
    int* d_boxes = nullptr;
    int* d_cell_box = nullptr;
    DevScalars* d_scal = nullptr;
    double *A = nullptr, *B = nullptr, *C = nullptr, *UL = nullptr, *UR = nullptr, *FX = nullptr;
    double *ulstar = nullptr, *urstar = nullptr, *gstar[3] = {nullptr, nullptr, nullptr};
    double* staging = nullptr;
    size_t staging_bytes = 0;
    // whole-box downloads: the copy of each converted slab runs on a second
    // stream while the next slab is converted
    static constexpr int kSlabs = 8;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t slab_ev[kSlabs + 1] = {};
    int coherent_host = -1;  // device reads host memory coherently (unknown until asked)
    MixedState mixed;
    // graph-captured step groups
    cudaGraphExec_t graph_exec = nullptr;
    int graph_steps = 0;
    long long launches = 0;
    EventProf* prof = nullptr;
    long long graph_launches = 0;
    AdjState* adj = nullptr;  // checkpoints and buffers of tj_forward / tj_backward
    TanState* tan = nullptr;  // buffers of tj_tangent
    GenAdj* gen = nullptr;    // the general reverse mode (configurations the 2-D adjoint does not cover)
    bool adj_general = false; // the last tj_forward took the general reverse mode
    double* cons = nullptr;   // conservation sums: partials, then the M + 4 results
};

namespace {

int fail(tj_ctx* c, int code, const std::string& msg)
{
    if (c) c->err = msg;
    return code;
}

#define TJ_CUDA(c, call)                                                                      \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return fail((c), TJ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// BoxList::maxSize (AMReX): power-of-two factoring, near-equal chunks chopped
// from the high end, one direction after another.
std::vector<int> max_size_boxes(const int* n, int dim, int mgs)
{
    std::vector<std::vector<int>> bl{{0, 0, 0, n[0] - 1, n[1] - 1, n[2] - 1}};
    for (int d = 0; d < dim; ++d) {
        std::vector<std::vector<int>> out;
        for (auto b : bl) {
            int len = b[3 + d] - b[d] + 1;
            if (len > mgs) {
                int ratio = 1, bs = mgs, nlen = len;
                while (bs % 2 == 0 && nlen % 2 == 0) { ratio *= 2; bs /= 2; nlen /= 2; }
                int numblk = nlen / bs + (nlen % bs ? 1 : 0), sz = nlen / numblk, ex = nlen % numblk;
                for (int k = 0; k < numblk - 1; ++k) {
                    int ksize = k < ex ? sz + 1 : sz;
                    int pos = b[3 + d] - ksize * ratio + 1;
                    auto up = b;
                    up[d] = pos;
                    b[3 + d] = pos - 1;
                    out.push_back(up);
                }
            }
            out.push_back(b);
        }
        bl.swap(out);
    }
    std::vector<int> flat;
    for (auto& b : bl) flat.insert(flat.end(), b.begin(), b.end());
    return flat;
}

void free_dev(tj_ctx* c)
{
    void* ps[] = {c->d_doms, c->d_boxes, c->d_cell_box, c->A, c->B, c->C, c->UL, c->UR, c->FX, c->ulstar, c->urstar,
                  c->gstar[0], c->gstar[1], c->gstar[2], c->staging};
    for (void* p : ps)
        if (p) cudaFree(p);
    c->d_doms = nullptr; c->d_boxes = nullptr; c->d_cell_box = nullptr;
    c->A = c->B = c->C = c->UL = c->UR = c->FX = c->ulstar = c->urstar = nullptr;
    c->gstar[0] = c->gstar[1] = c->gstar[2] = nullptr;
    c->staging = nullptr;
    c->staging_bytes = 0;
    mixed_free(c->mixed);
    if (c->graph_exec) { cudaGraphExecDestroy(c->graph_exec); c->graph_exec = nullptr; }
    adj_destroy(c->adj);
    tan_destroy(c->tan);
    c->tan = nullptr;
    gen_destroy(c->gen);
    c->gen = nullptr;
    c->adj = nullptr;
}

Fp64Bufs bufs(tj_ctx* c)
{
    Fp64Bufs b;
    b.A = c->A; b.B = c->B; b.C = c->C; b.UL = c->UL; b.UR = c->UR; b.FX = c->FX;
    b.ulstar = c->ulstar; b.urstar = c->urstar;
    for (int d = 0; d < 3; ++d) { b.gstar[d] = c->gstar[d]; b.nftot[d] = c->nftot[d]; }
    b.cell_box = c->d_cell_box; b.boxes = c->d_boxes; b.doms = c->d_doms; b.scal = c->d_scal;
    b.ntot = c->ntot; b.ndom = (int)c->doms.size();
    return b;
}

// both fused precisions run the fused kernels
bool is_mixed(const tj_ctx* c)
{
    return c->params.precision == TJ_PRECISION_MIXED || c->params.precision == TJ_PRECISION_FUSED64;
}

// Upload the box table and the cell -> box map (geometry changes only).
int sync_boxes(tj_ctx* c)
{
    c->geometry_dirty = false;
    std::vector<int> flat;
    std::vector<int> cell_box(c->ntot);
    for (size_t q = 0; q < c->doms.size(); ++q) {
        DevDomain& D = c->doms[q];
        D.box_off = (int)(flat.size() / 6);
        D.nbox = (int)(c->boxes[q].size() / 6);
        flat.insert(flat.end(), c->boxes[q].begin(), c->boxes[q].end());
        for (int b = 0; b < D.nbox; ++b) {
            const int* B = &c->boxes[q][6 * b];
            for (int k = B[2]; k <= B[5]; ++k)
                for (int j = B[1]; j <= B[4]; ++j)
                    for (int i = B[0]; i <= B[3]; ++i)
                        cell_box[D.off + i + (long long)D.n[0] * (j + (long long)D.n[1] * k)] = b;
        }
    }
    if (c->d_boxes) cudaFree(c->d_boxes);
    TJ_CUDA(c, cudaMalloc(&c->d_boxes, sizeof(int) * std::max<size_t>(flat.size(), 6)));
    TJ_CUDA(c, cudaMemcpy(c->d_boxes, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice));
    TJ_CUDA(c, cudaMemcpy(c->d_cell_box, cell_box.data(), sizeof(int) * c->ntot, cudaMemcpyHostToDevice));
    TJ_CUDA(c, cudaMemcpy(c->d_doms, c->doms.data(), sizeof(DevDomain) * c->doms.size(), cudaMemcpyHostToDevice));
    if (c->graph_exec) { cudaGraphExecDestroy(c->graph_exec); c->graph_exec = nullptr; }
    if (is_mixed(c)) return mixed_set_boxes(c->mixed, c->P, c->doms, c->boxes, c->stream);
    return TJ_OK;
}

int need_state(tj_ctx* c)
{
    if (c->doms.empty() || !c->A) return fail(c, TJ_ERR_STATE, "no domain set (tj_set_domains)");
    if (c->geometry_dirty) {
        TJ_CUDA(c, cudaStreamSynchronize(c->stream));
        int e = sync_boxes(c);
        if (e) return e;
    }
    return TJ_OK;
}

// The FP64 carried state is about to be read: bring it up to date.
void a_sync(tj_ctx* c)
{
    if (is_mixed(c) && !c->a_current) {
        Fp64Bufs b = bufs(c);
        c->launches += mixed_to_fp64(c->mixed, c->P, b, c->stream);
        c->a_current = true;
    }
}

// The fused kernels are about to run: bring their state up to date (and arm
// the CFL minimum of the next step).
void x_sync(tj_ctx* c)
{
    if (is_mixed(c) && !c->x_current) {
        Fp64Bufs b = bufs(c);
        c->launches += mixed_from_fp64(c->mixed, c->P, b, c->stream);
        c->x_current = true;
    }
}

// The FP64 carried state was written.
void a_written(tj_ctx* c)
{
    c->a_current = true;
    if (is_mixed(c)) c->x_current = false;
}

int check_status(tj_ctx* c)
{
    DevScalars s;
    TJ_CUDA(c, cudaMemcpyAsync(&s, c->d_scal, sizeof s, cudaMemcpyDeviceToHost, c->stream));
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    if (s.status != 0) {
        const char* what = s.status == TJ_ERR_WAVESPEED ? "NaN in wave speeds (hllc.cpp:169-200)"
                           : s.status == TJ_ERR_ALPHA   ? "error in scaling volume fractions (boxaccesscellarray.cpp:553-588)"
                           : s.status == TJ_ERR_PLASTIC ? "divide by zero in the plastic update (plastic.cpp:189-193)"
                           : s.status == TJ_ERR_NAN     ? "NaN found in the state (main.cpp:183-187)"
                           : s.status == TJ_ERR_ROOT    ? "no sign change in the mixture root bisection "
                                                          "(equationofstate.cpp:327-335)"
                                                        : "device error";
        return fail(c, s.status, what);
    }
    return TJ_OK;
}

// One full iteration of main.cpp:121-191, device-side dt and t.
int issue_step(tj_ctx* c)
{
    Fp64Bufs b = bufs(c);
    int n = 0;
    Prof* pr = c->prof;
    if (is_mixed(c)) {
        n += mixed_step(c->mixed, c->P, b, c->stream, pr);
    } else {
        n += fp64_cfl(c->P, b, c->A, c->stream, pr);
        n += fp64_dt_finalize(c->P, b, 1, c->stream);
        n += fp64_stage(c->P, b, c->A, c->B, 0, c->stream, pr);
        n += fp64_stage(c->P, b, c->B, c->C, 1, c->stream, pr);
        n += fp64_step_end(b, c->stream);
    }
    c->launches += n;
    return TJ_OK;
}

}  // namespace

extern "C" {

int tj_create(const tj_params* p, tj_ctx** out)
{
    if (!p || !out) return TJ_ERR_ARG;
    *out = nullptr;
    tj_ctx* c = new tj_ctx();
    c->params = *p;
    auto bad = [&](const char* m) {
        std::fprintf(stderr, "tj_create: %s\n", m);
        delete c;
        return TJ_ERR_ARG;
    };
    if (p->dim < 1 || p->dim > 3) return bad("dim must be 1, 2 or 3");
    if (p->n_materials < 1 || p->n_materials > TJ_MAX_MATERIALS) return bad("n_materials out of range");
    if (p->n_mixtures < 0 || p->n_mixtures > 1)
        return bad("n_mixtures must be 0 or 1: the reference indexes every mixture at mixtureIndex 0 "
                   "(initialise.cpp:187, boxaccesscellarray.cpp:43-47)");
    {
        int nmixeos = 0;
        for (int m = 0; m < p->n_materials && m < TJ_MAX_MATERIALS; ++m) nmixeos += p->materials[m].eos == TJ_EOS_MIXTURE;
        if (nmixeos != p->n_mixtures) return bad("n_mixtures must equal the number of TJ_EOS_MIXTURE materials");
        if (p->n_mixtures && p->materials[0].eos != TJ_EOS_MIXTURE)
            return bad("the mixture must be material 0 (the reference's Cell maps mixture 0 to material 0, "
                       "cell.cpp:95-97, hllc.cpp:26-29)");
        if (p->n_mixtures && p->materials[0].phase != TJ_PHASE_FLUID) return bad("a mixture is a fluid (initialise.cpp:158-178)");
        if (p->n_mixtures && p->SOLID) return bad("mixtures with SOLID are not supported");
    }
    if (p->RADIAL && p->SOLID && !p->PLASTIC)
        return bad("RADIAL with elastic solids is not supported: the source term reads the RK2-averaged stress "
                   "(hllc.cpp:705, radial.cpp:23), which the carried state does not hold");
    if (p->nghost < 2) return bad("nghost must be >= 2");
    if (p->THINC && p->dim == 3) return bad("THINC is 1-D/2-D only in the reference (thinc.cpp:116-127)");
    if (p->THINC && !p->MUSCL) return bad("THINC needs MUSCL");
    if (p->THINC && p->SOLID) return bad("THINC with SOLID is not supported");
    if (p->PLASTIC && !p->SOLID) return bad("PLASTIC needs SOLID");
    if (p->PLASTIC > 1) return bad("only PLASTIC=1 (radial return) is supported");
    int any_solid = 0;
    for (int m = 0; m < p->n_materials; ++m) {
        const tj_material& mt = p->materials[m];
        if (mt.eos < 0 || mt.eos > TJ_EOS_MIXTURE) return bad("unknown EOS");
        int need = mt.eos == TJ_EOS_MIEGRUNEISEN ? 4 : mt.eos == TJ_EOS_ROMENSKII ? 9 : mt.eos == TJ_EOS_WILKINS ? 11 : 8;
        if (mt.nparams < need) return bad("too few EOS parameters");
        if (mt.phase == TJ_PHASE_SOLID) {
            any_solid = 1;
            if (mt.eos == TJ_EOS_MIEGRUNEISEN || mt.eos == TJ_EOS_MIXTURE) return bad("a solid needs a solid EOS");
        }
    }
    if (p->SOLID && !any_solid) return bad("SOLID needs a solid material");
    if (p->precision != TJ_PRECISION_FP64 && p->precision != TJ_PRECISION_MIXED && p->precision != TJ_PRECISION_FUSED64)
        return bad("unknown precision");
    if (p->precision != TJ_PRECISION_FP64 && !mixed_supported(*p))
        return bad("the fused precisions support fluids with the stiffened-gas EOS in 2-D, and in 3-D without THINC "
                   "in binary32 only");
    make_layouts(*p, c->P);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return bad("no CUDA device");
    if (cudaMalloc(&c->d_scal, sizeof(DevScalars)) != cudaSuccess) return bad("cudaMalloc failed");
    DevScalars s;
    std::memset(&s, 0, sizeof s);
    s.t_end = 1e300;
    s.dtmin_bits = 0x7FEFFFFFFFFFFFFFull;
    cudaMemcpy(c->d_scal, &s, sizeof s, cudaMemcpyHostToDevice);
    *out = c;
    return TJ_OK;
}

int tj_destroy(tj_ctx* c)
{
    if (!c) return TJ_OK;
    cudaStreamSynchronize(c->stream);
    free_dev(c);
    delete c->prof;
    c->prof = nullptr;
    if (c->d_scal) cudaFree(c->d_scal);
    if (c->cons) cudaFree(c->cons);
    for (cudaEvent_t& e : c->slab_ev)
        if (e) cudaEventDestroy(e);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return TJ_OK;
}

int tj_last_error(const tj_ctx* c, char* buf, unsigned long len)
{
    if (!c || !buf || len == 0) return TJ_ERR_ARG;
    std::snprintf(buf, len, "%s", c->err.c_str());
    return TJ_OK;
}

int tj_ncomp(const tj_ctx* c) { return c ? c->P.NCOMP : TJ_ERR_ARG; }

int tj_set_domains(tj_ctx* c, int nd, const int* n_cells, const double* dim_l)
{
    if (!c || nd < 1 || !n_cells || !dim_l) return fail(c, TJ_ERR_ARG, "bad domain arguments");
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    free_dev(c);
    c->doms.assign(nd, DevDomain());
    c->boxes.assign(nd, std::vector<int>());
    long long off = 0, foff[3] = {0, 0, 0};
    for (int q = 0; q < nd; ++q) {
        DevDomain& D = c->doms[q];
        for (int k = 0; k < 3; ++k) {
            D.n[k] = k < c->P.dim ? n_cells[3 * q + k] : 1;
            if (D.n[k] < 1) return fail(c, TJ_ERR_ARG, "n_cells must be >= 1");
            if (k < c->P.dim && D.n[k] < 1) return fail(c, TJ_ERR_ARG, "empty domain");
            D.dx[k] = (k < c->P.dim ? dim_l[3 * q + k] : (dim_l[3 * q + k] > 0 ? dim_l[3 * q + k] : 1.0)) / (double)D.n[k];
        }
        D.off = off;
        off += (long long)D.n[0] * D.n[1] * D.n[2];
        for (int d = 0; d < 3; ++d) {
            D.foff[d] = foff[d];
            long long nf = (long long)(D.n[0] + (d == 0)) * (D.n[1] + (d == 1)) * (D.n[2] + (d == 2));
            foff[d] += nf;
        }
        c->boxes[q] = {0, 0, 0, D.n[0] - 1, D.n[1] - 1, D.n[2] - 1};
    }
    c->ntot = off;
    for (int d = 0; d < 3; ++d) c->nftot[d] = foff[d];
    const DevParams& P = c->P;
    size_t nt = (size_t)c->ntot;
    TJ_CUDA(c, cudaMalloc(&c->d_doms, sizeof(DevDomain) * nd));
    TJ_CUDA(c, cudaMalloc(&c->d_cell_box, sizeof(int) * nt));
    if (is_mixed(c)) {
        int e = mixed_alloc(c->mixed, P, c->doms, c->ntot, c->nftot, c->stream);
        if (e) return fail(c, e, "mixed-precision allocation failed");
        // the FP64 buffers double as the mixed path's conversion staging
        TJ_CUDA(c, cudaMalloc(&c->A, sizeof(double) * P.NS * nt));
        TJ_CUDA(c, cudaMemset(c->A, 0, sizeof(double) * P.NS * nt));
    } else {
        size_t fmax = (size_t)std::max(c->nftot[0], std::max(c->nftot[1], c->nftot[2]));
        TJ_CUDA(c, cudaMalloc(&c->A, sizeof(double) * P.NS * nt));
        TJ_CUDA(c, cudaMalloc(&c->B, sizeof(double) * P.NS * nt));
        TJ_CUDA(c, cudaMalloc(&c->C, sizeof(double) * P.NS * nt));
        TJ_CUDA(c, cudaMalloc(&c->UL, sizeof(double) * P.NF * nt));
        TJ_CUDA(c, cudaMalloc(&c->UR, sizeof(double) * P.NF * nt));
        TJ_CUDA(c, cudaMalloc(&c->FX, sizeof(double) * P.NX * fmax));
        TJ_CUDA(c, cudaMemset(c->A, 0, sizeof(double) * P.NS * nt));
        TJ_CUDA(c, cudaMemset(c->B, 0, sizeof(double) * P.NS * nt));
        TJ_CUDA(c, cudaMemset(c->C, 0, sizeof(double) * P.NS * nt));
        if (P.thinc) {
            TJ_CUDA(c, cudaMalloc(&c->ulstar, sizeof(double) * P.M * nt));
            TJ_CUDA(c, cudaMalloc(&c->urstar, sizeof(double) * P.M * nt));
            TJ_CUDA(c, cudaMemset(c->ulstar, 0, sizeof(double) * P.M * nt));
            TJ_CUDA(c, cudaMemset(c->urstar, 0, sizeof(double) * P.M * nt));
            for (int d = 0; d < P.dim; ++d) {
                TJ_CUDA(c, cudaMalloc(&c->gstar[d], sizeof(double) * P.M * c->nftot[d]));
                TJ_CUDA(c, cudaMemset(c->gstar[d], 0, sizeof(double) * P.M * c->nftot[d]));
            }
        }
    }
    c->a_current = c->x_current = true;  // both copies start zero
    int e = sync_boxes(c);
    if (e) return e;
    return tj_set_time(c, 0.0, 0);
}

int tj_set_boxes(tj_ctx* c, int q, int nbox, const int* lohi)
{
    if (!c || q < 0 || q >= (int)c->doms.size() || nbox < 1 || !lohi) return fail(c, TJ_ERR_ARG, "bad box arguments");
    const DevDomain& D = c->doms[q];
    std::vector<int> cover((size_t)D.n[0] * D.n[1] * D.n[2], 0);
    for (int b = 0; b < nbox; ++b) {
        const int* B = lohi + 6 * b;
        for (int k = 0; k < 3; ++k)
            if (B[k] < 0 || B[3 + k] >= D.n[k] || B[k] > B[3 + k]) return fail(c, TJ_ERR_ARG, "box outside the domain");
        for (int k = B[2]; k <= B[5]; ++k)
            for (int j = B[1]; j <= B[4]; ++j)
                for (int i = B[0]; i <= B[3]; ++i) cover[i + (size_t)D.n[0] * (j + (size_t)D.n[1] * k)]++;
    }
    for (int v : cover)
        if (v != 1) return fail(c, TJ_ERR_ARG, "boxes must tile the domain exactly once");
    c->boxes[q].assign(lohi, lohi + 6 * nbox);
    c->geometry_dirty = true;  // uploaded before the next operation that needs it
    return TJ_OK;
}

int tj_set_max_grid_size(tj_ctx* c, int q, int mgs)
{
    if (!c || q < 0 || q >= (int)c->doms.size() || mgs < 1) return fail(c, TJ_ERR_ARG, "bad max_grid_size");
    std::vector<int> bl = max_size_boxes(c->doms[q].n, c->P.dim, mgs);
    return tj_set_boxes(c, q, (int)(bl.size() / 6), bl.data());
}

int tj_num_boxes(const tj_ctx* c, int q)
{
    if (!c || q < 0 || q >= (int)c->doms.size()) return TJ_ERR_ARG;
    return (int)(c->boxes[q].size() / 6);
}

int tj_get_box(const tj_ctx* c, int q, int b, int* lohi)
{
    if (!c || q < 0 || q >= (int)c->doms.size() || b < 0 || b >= (int)(c->boxes[q].size() / 6) || !lohi) return TJ_ERR_ARG;
    std::memcpy(lohi, &c->boxes[q][6 * b], 6 * sizeof(int));
    return TJ_OK;
}

int tj_num_cells(const tj_ctx* c, long long* n)
{
    if (!c || !n) return TJ_ERR_ARG;
    *n = c->ntot;
    return TJ_OK;
}

static int ensure_staging(tj_ctx* c, size_t bytes)
{
    if (c->staging_bytes >= bytes) return TJ_OK;
    if (c->staging) cudaFree(c->staging);
    c->staging = nullptr;
    TJ_CUDA(c, cudaMalloc(&c->staging, bytes));
    c->staging_bytes = bytes;
    return TJ_OK;
}

// The device address of a host buffer the conversion kernels may read and
// write in place, or null. Taken when the device accesses host memory
// coherently (a Grace host over NVLink-C2C: any valid host address is legal
// there) and both ends of the buffer are page-locked and mapped at the same
// offset: the kernels then move each byte across the link once, at the
// link's rate, with no staging copy and no separate conversion pass. A buffer
// the device writes must also come from cudaHostAlloc (cudaHostGetFlags
// answers for it): registered memory may be mapped read-only to the device.
static double* mapped_view(tj_ctx* c, double* host, size_t bytes, bool device_writes)
{
    if (c->coherent_host < 0) {
        int dev = 0, v = 0;
        c->coherent_host = cudaGetDevice(&dev) == cudaSuccess &&
                           cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess && v == 1;
    }
    if (!c->coherent_host || bytes == 0) return nullptr;
    cudaPointerAttributes a{}, z{};
    const char* last = reinterpret_cast<const char*>(host) + bytes - 1;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess || cudaPointerGetAttributes(&z, last) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || z.type != cudaMemoryTypeHost || !a.devicePointer ||
        static_cast<const char*>(z.devicePointer) != static_cast<const char*>(a.devicePointer) + (bytes - 1))
        return nullptr;
    if (device_writes) {
        unsigned int flags = 0;
        if (cudaHostGetFlags(&flags, host) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
    }
    return static_cast<double*>(a.devicePointer);
}

static int exchange(tj_ctx* c, int q, const int* bx, double* host, int ncomp, int ngrow, bool up)
{
    int e = need_state(c);
    if (e) return e;
    if (ncomp != c->P.NCOMP) return fail(c, TJ_ERR_ARG, "ncomp must equal tj_ncomp()");
    int dim = c->P.dim;
    int ld_i = bx[3] - bx[0] + 1 + 2 * ngrow;
    int ld_j = bx[4] - bx[1] + 1 + (dim > 1 ? 2 * ngrow : 0);
    int ld_k = bx[5] - bx[2] + 1 + (dim > 2 ? 2 * ngrow : 0);
    long long cs = (long long)ld_i * ld_j * ld_k;
    size_t bytes = sizeof(double) * ncomp * cs;
    Fp64Bufs b = bufs(c);
    // an upload of the whole of the only domain replaces the state entirely;
    // any other keeps the cells outside the box
    const DevDomain& Dq = c->doms[q];
    const bool whole = c->doms.size() == 1 && bx[0] == 0 && bx[1] == 0 && bx[2] == 0 && bx[3] == Dq.n[0] - 1 &&
                       bx[4] == Dq.n[1] - 1 && bx[5] == Dq.n[2] - 1;
    if (double* dv = mapped_view(c, host, bytes, !up)) {
        // in place: the kernels read (write) the caller's page-locked buffer
        if (up) {
            if (!whole) a_sync(c);
            // the fused 2-D state is filled in the same pass (no conversion
            // before the next step)
            const int r = whole && ngrow == 0 && is_mixed(c) ? mixed_from_ap(c->mixed, c->P, b, dv, c->stream) : -1;
            if (r >= 0) {
                c->launches += r;
                c->a_current = c->x_current = true;
            } else {
                c->launches += fp64_ap_to_state(c->P, b, q, bx, dv, ld_i, ld_j, ld_k, cs, ngrow, c->A, c->stream);
                a_written(c);
            }
        } else {
            a_sync(c);
            c->launches += fp64_state_to_ap(c->P, b, q, bx, c->A, dv, ld_i, ld_j, ld_k, cs, ngrow, c->stream);
        }
        TJ_CUDA(c, cudaStreamSynchronize(c->stream));
        TJ_CUDA(c, cudaGetLastError());
        return TJ_OK;
    }
    e = ensure_staging(c, bytes);
    if (e) return e;
    if (up) {
        if (!whole) a_sync(c);
        // only the component planes the carried state is built from cross the
        // link (k_ap_to_state reads no other)
        const DevParams& P = c->P;
        int rng[5][2] = {{P.A_ALPHA, P.A_P + 1}, {-1, -1}, {-1, -1}, {-1, -1}, {-1, -1}};
        if (P.nmix) { rng[1][0] = P.A_RMIX; rng[1][1] = P.A_ARL + 1; }
        if (P.solid) { rng[2][0] = P.A_V; rng[2][1] = P.A_V + 9; rng[3][0] = P.A_HJ2; rng[3][1] = P.A_HJ2 + 1; }
        if (P.plastic) { rng[4][0] = P.A_EPS; rng[4][1] = P.A_ARE + P.M; }
        for (auto& r : rng)
            if (r[0] >= 0)
                TJ_CUDA(c, cudaMemcpyAsync(c->staging + (size_t)r[0] * cs, host + (size_t)r[0] * cs,
                                           sizeof(double) * (size_t)(r[1] - r[0]) * cs, cudaMemcpyDefault, c->stream));
        c->launches += fp64_ap_to_state(c->P, b, q, bx, c->staging, ld_i, ld_j, ld_k, cs, ngrow, c->A, c->stream);
        a_written(c);
        TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    } else {
        a_sync(c);
        if (ngrow == 0 && cs >= (1 << 16)) {
            // slab k's components are rows [t0, t1) of every plane: one 2-D copy
            // per slab, overlapped with the conversion of slab k + 1
            if (!c->copy_stream) {
                TJ_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
                for (cudaEvent_t& e : c->slab_ev) TJ_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            }
            const int K = tj_ctx::kSlabs;
            for (int k = 0; k < K; ++k) {
                const long long t0 = cs * k / K, t1 = cs * (k + 1) / K;
                c->launches += fp64_state_to_ap(c->P, b, q, bx, c->A, c->staging, ld_i, ld_j, ld_k, cs, 0, c->stream, t0, t1);
                TJ_CUDA(c, cudaEventRecord(c->slab_ev[k], c->stream));
                TJ_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->slab_ev[k], 0));
                TJ_CUDA(c, cudaMemcpy2DAsync(host + t0, sizeof(double) * (size_t)cs, c->staging + t0,
                                             sizeof(double) * (size_t)cs, sizeof(double) * (size_t)(t1 - t0), ncomp,
                                             cudaMemcpyDefault, c->copy_stream));
            }
            TJ_CUDA(c, cudaEventRecord(c->slab_ev[K], c->copy_stream));
            TJ_CUDA(c, cudaStreamWaitEvent(c->stream, c->slab_ev[K], 0));
        } else {
            if (ngrow > 0) TJ_CUDA(c, cudaMemcpyAsync(c->staging, host, bytes, cudaMemcpyDefault, c->stream));
            c->launches += fp64_state_to_ap(c->P, b, q, bx, c->A, c->staging, ld_i, ld_j, ld_k, cs, ngrow, c->stream);
            TJ_CUDA(c, cudaMemcpyAsync(host, c->staging, bytes, cudaMemcpyDefault, c->stream));
        }
        TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    TJ_CUDA(c, cudaGetLastError());
    return TJ_OK;
}

int tj_upload_state(tj_ctx* c, int q, int box, const double* fab, int ncomp, int ngrow)
{
    if (!c || q < 0 || q >= (int)c->doms.size() || box < 0 || box >= (int)(c->boxes[q].size() / 6) || !fab || ngrow < 0)
        return fail(c, TJ_ERR_ARG, "bad upload arguments");
    return exchange(c, q, &c->boxes[q][6 * box], const_cast<double*>(fab), ncomp, ngrow, true);
}

int tj_download_state(tj_ctx* c, int q, int box, double* fab, int ncomp, int ngrow)
{
    if (!c || q < 0 || q >= (int)c->doms.size() || box < 0 || box >= (int)(c->boxes[q].size() / 6) || !fab || ngrow < 0)
        return fail(c, TJ_ERR_ARG, "bad download arguments");
    return exchange(c, q, &c->boxes[q][6 * box], fab, ncomp, ngrow, false);
}

int tj_upload_domain(tj_ctx* c, int q, const double* data)
{
    if (!c || q < 0 || q >= (int)c->doms.size() || !data) return fail(c, TJ_ERR_ARG, "bad upload arguments");
    const DevDomain& D = c->doms[q];
    int bx[6] = {0, 0, 0, D.n[0] - 1, D.n[1] - 1, D.n[2] - 1};
    return exchange(c, q, bx, const_cast<double*>(data), c->P.NCOMP, 0, true);
}

int tj_download_domain(tj_ctx* c, int q, double* data)
{
    if (!c || q < 0 || q >= (int)c->doms.size() || !data) return fail(c, TJ_ERR_ARG, "bad download arguments");
    const DevDomain& D = c->doms[q];
    int bx[6] = {0, 0, 0, D.n[0] - 1, D.n[1] - 1, D.n[2] - 1};
    return exchange(c, q, bx, data, c->P.NCOMP, 0, false);
}

int tj_set_primitive(tj_ctx* c, int q, const double* prim)
{
    if (!c || q < 0 || q >= (int)c->doms.size() || !prim) return fail(c, TJ_ERR_ARG, "bad primitive arguments");
    int e = need_state(c);
    if (e) return e;
    const DevDomain& D = c->doms[q];
    int nprim = 2 * c->P.M + 4 + (c->P.solid ? 9 : 0) + (c->P.plastic ? c->P.M : 0) + c->P.nmix;
    size_t bytes = sizeof(double) * nprim * (size_t)D.n[0] * D.n[1] * D.n[2];
    e = ensure_staging(c, bytes);
    if (e) return e;
    TJ_CUDA(c, cudaMemcpyAsync(c->staging, prim, bytes, cudaMemcpyDefault, c->stream));
    a_sync(c);
    Fp64Bufs b = bufs(c);
    c->launches += fp64_prim_to_state(c->P, b, q, c->staging, c->A, c->stream);
    a_written(c);
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    TJ_CUDA(c, cudaGetLastError());
    return TJ_OK;
}

int tj_compute_dt(tj_ctx* c, double* dt)
{
    if (!c || !dt) return TJ_ERR_ARG;
    int e = need_state(c);
    if (e) return e;
    Fp64Bufs b = bufs(c);
    c->launches += fp64_set_dt(b, 0.0, c->stream);
    if (is_mixed(c)) {
        x_sync(c);
        c->launches += mixed_compute_dt(c->mixed, c->P, b, c->stream);
        c->launches += fp64_dt_finalize(c->P, b, 0, c->stream);
        c->launches += mixed_compute_dt(c->mixed, c->P, b, c->stream);  // re-arm for the next step
    } else {
        c->launches += fp64_cfl(c->P, b, c->A, c->stream);
        c->launches += fp64_dt_finalize(c->P, b, 0, c->stream);
    }
    DevScalars s;
    TJ_CUDA(c, cudaMemcpyAsync(&s, c->d_scal, sizeof s, cudaMemcpyDeviceToHost, c->stream));
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    *dt = c->P.cfl * s.dtmin_raw;
    return TJ_OK;
}

int tj_advance(tj_ctx* c, double dt)
{
    if (!c) return TJ_ERR_ARG;
    int e = need_state(c);
    if (e) return e;
    Fp64Bufs b = bufs(c);
    c->launches += fp64_set_dt(b, dt, c->stream);
    if (is_mixed(c)) return fail(c, TJ_ERR_ARG, "tj_advance alone is FP64-only; use tj_step/tj_run in mixed precision");
    // advance() alone: both stages and the average (finish mode 2), without
    // the post-advance operators, which have their own entry points.
    c->launches += fp64_stage(c->P, b, c->A, c->B, 0, c->stream);
    c->launches += fp64_stage(c->P, b, c->B, c->C, 2, c->stream);
    TJ_CUDA(c, cudaGetLastError());
    return check_status(c);
}

int tj_advance_stage(tj_ctx* c, int stage, double dt)
{
    if (!c || (stage != 0 && stage != 1)) return TJ_ERR_ARG;
    int e = need_state(c);
    if (e) return e;
    if (is_mixed(c)) return fail(c, TJ_ERR_ARG, "tj_advance_stage is FP64-only");
    Fp64Bufs b = bufs(c);
    const size_t bytes = sizeof(double) * (size_t)c->P.NS * (size_t)c->ntot;
    c->launches += fp64_set_dt(b, dt, c->stream);
    if (stage == 0) {
        // U^n is kept in C for the second stage's average; the state becomes
        // U1 = HLLCadvance(U^n)
        TJ_CUDA(c, cudaMemcpyAsync(c->C, c->A, bytes, cudaMemcpyDeviceToDevice, c->stream));
        c->launches += fp64_stage(c->P, b, c->A, c->B, 0, c->stream);
        TJ_CUDA(c, cudaMemcpyAsync(c->A, c->B, bytes, cudaMemcpyDeviceToDevice, c->stream));
        c->stage0_done = true;
    } else {
        if (!c->stage0_done) return fail(c, TJ_ERR_STATE, "tj_advance_stage(1) follows tj_advance_stage(0)");
        // U2 = HLLCadvance(U1), then U1 = U^n/2 + U2/2 (hllc.cpp:701-705)
        Fp64Bufs bb = b;
        bb.A = c->C;
        c->launches += fp64_stage(c->P, bb, c->A, c->B, 2, c->stream);
        TJ_CUDA(c, cudaMemcpyAsync(c->A, c->C, bytes, cudaMemcpyDeviceToDevice, c->stream));
        c->stage0_done = false;
    }
    TJ_CUDA(c, cudaGetLastError());
    return check_status(c);
}

static int cell_op(tj_ctx* c, int op, double dt = 0.0)
{
    int e = need_state(c);
    if (e) return e;
    Fp64Bufs b = bufs(c);
    a_sync(c);
    c->launches += fp64_cell_op(c->P, b, c->A, nullptr, op, c->stream, dt);
    if (op != OP_NAN) a_written(c);
    TJ_CUDA(c, cudaGetLastError());
    return check_status(c);
}

int tj_plastic_update(tj_ctx* c, double dt)
{
    (void)dt;
    if (!c) return TJ_ERR_ARG;
    if (!c->P.plastic) return TJ_OK;
    return cell_op(c, OP_PLASTIC);
}
int tj_reactive_update(tj_ctx* c, double dt)
{
    if (!c) return TJ_ERR_ARG;
    if (!(dt >= 0.0)) return fail(c, TJ_ERR_ARG, "tj_reactive_update: dt must be >= 0");
    if (!c->P.nmix) return TJ_OK;  // reactive.cpp:64
    return cell_op(c, OP_REACTIVE, dt);
}

int tj_geometric_source(tj_ctx* c, double dt)
{
    if (!c) return TJ_ERR_ARG;
    if (!(dt >= 0.0)) return fail(c, TJ_ERR_ARG, "tj_geometric_source: dt must be >= 0");
    return cell_op(c, OP_RADIAL, dt);
}
int tj_cleanup_v(tj_ctx* c) { return c ? (c->P.solid ? cell_op(c, OP_CLEAN_V) : TJ_OK) : TJ_ERR_ARG; }
int tj_cleanup_alpha(tj_ctx* c) { return c ? cell_op(c, OP_CLEAN_ALPHA) : TJ_ERR_ARG; }
int tj_cons_to_prim(tj_ctx* c) { return c ? cell_op(c, OP_C2P) : TJ_ERR_ARG; }
int tj_prim_to_cons(tj_ctx* c) { return c ? cell_op(c, OP_P2C) : TJ_ERR_ARG; }

int tj_contains_nan(tj_ctx* c, int* flag)
{
    if (!c || !flag) return TJ_ERR_ARG;
    int e = need_state(c);
    if (e) return e;
    TJ_CUDA(c, cudaMemsetAsync(&c->d_scal->nan_flag, 0, sizeof(int), c->stream));
    Fp64Bufs b = bufs(c);
    a_sync(c);
    c->launches += fp64_cell_op(c->P, b, c->A, nullptr, OP_NAN, c->stream);
    DevScalars s;
    TJ_CUDA(c, cudaMemcpyAsync(&s, c->d_scal, sizeof s, cudaMemcpyDeviceToHost, c->stream));
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    TJ_CUDA(c, cudaMemsetAsync(&c->d_scal->nan_flag, 0, sizeof(int), c->stream));
    *flag = s.nan_flag ? 1 : 0;
    return TJ_OK;
}

int tj_conservation_sums(tj_ctx* c, double* sums)
{
    if (!c || !sums) return TJ_ERR_ARG;
    int e = need_state(c);
    if (e) return e;
    const int nv = c->P.M + 4;
    if (!c->cons) TJ_CUDA(c, cudaMalloc(&c->cons, sizeof(double) * (size_t)(kConsPartials + 1) * nv));
    a_sync(c);
    Fp64Bufs b = bufs(c);
    double* out = c->cons + (size_t)kConsPartials * nv;
    c->launches += fp64_conservation(c->P, b, c->A, c->cons, out, c->stream);
    TJ_CUDA(c, cudaMemcpyAsync(sums, out, sizeof(double) * nv, cudaMemcpyDeviceToHost, c->stream));
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    TJ_CUDA(c, cudaGetLastError());
    return TJ_OK;
}

int tj_download_component(tj_ctx* c, int q, int comp, double* data)
{
    if (!c || q < 0 || q >= (int)c->doms.size() || !data || comp < 0 || comp >= c->P.NCOMP)
        return fail(c, TJ_ERR_ARG, "bad component download arguments");
    int e = need_state(c);
    if (e) return e;
    const DevDomain& D = c->doms[q];
    const size_t bytes = sizeof(double) * (size_t)D.n[0] * D.n[1] * D.n[2];
    double* dst = mapped_view(c, data, bytes, true);
    if (!dst) {
        e = ensure_staging(c, bytes);
        if (e) return e;
        dst = c->staging;
    }
    a_sync(c);
    Fp64Bufs b = bufs(c);
    c->launches += fp64_state_component(c->P, b, q, c->A, comp, dst, c->stream);
    if (dst == c->staging) TJ_CUDA(c, cudaMemcpyAsync(data, dst, bytes, cudaMemcpyDeviceToHost, c->stream));
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    TJ_CUDA(c, cudaGetLastError());
    return TJ_OK;
}

int tj_set_time(tj_ctx* c, double t, int n)
{
    if (!c) return TJ_ERR_ARG;
    DevScalars s;
    TJ_CUDA(c, cudaMemcpyAsync(&s, c->d_scal, sizeof s, cudaMemcpyDeviceToHost, c->stream));
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    s.t = t;
    s.n = n;
    s.done = 0;
    s.status = 0;
    s.nan_flag = 0;
    s.dtmin_bits = 0x7FEFFFFFFFFFFFFFull;
    TJ_CUDA(c, cudaMemcpyAsync(c->d_scal, &s, sizeof s, cudaMemcpyHostToDevice, c->stream));
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    return TJ_OK;
}

int tj_get_time(tj_ctx* c, double* t, int* n, double* last_dt)
{
    if (!c) return TJ_ERR_ARG;
    DevScalars s;
    TJ_CUDA(c, cudaMemcpyAsync(&s, c->d_scal, sizeof s, cudaMemcpyDeviceToHost, c->stream));
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    if (t) *t = s.t;
    if (n) *n = s.n;
    if (last_dt) *last_dt = s.dt;
    return TJ_OK;
}

static int set_t_end(tj_ctx* c, double t_end)
{
    // t_end lives in the scalars block; a tiny host->device write of one field
    TJ_CUDA(c, cudaMemcpyAsync(&c->d_scal->t_end, &t_end, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    return TJ_OK;
}

int tj_step(tj_ctx* c, double t_end)
{
    if (!c) return TJ_ERR_ARG;
    int e = need_state(c);
    if (e) return e;
    e = set_t_end(c, t_end);
    if (e) return e;
    x_sync(c);
    issue_step(c);
    if (is_mixed(c)) c->a_current = false;
    TJ_CUDA(c, cudaGetLastError());
    return TJ_OK;
}

int tj_run(tj_ctx* c, int nsteps, double t_end, int* steps_done, double* t_out)
{
    if (!c || nsteps < 0) return TJ_ERR_ARG;
    int e = need_state(c);
    if (e) return e;
    e = set_t_end(c, t_end);
    if (e) return e;
    int n0 = 0;
    double t0 = 0;
    e = tj_get_time(c, &t0, &n0, nullptr);
    if (e) return e;
    x_sync(c);  // outside any capture
    if (is_mixed(c) && nsteps > 0) c->a_current = false;
    const int group = 20;
    long long per_group = 0;
    if (!c->graph_exec || c->graph_steps != group) {
        if (c->graph_exec) { cudaGraphExecDestroy(c->graph_exec); c->graph_exec = nullptr; }
        cudaGraph_t g;
        long long before = c->launches;
        if (c->prof) {
            c->prof->collect_direct();
            c->prof->reserve((size_t)group * 64 + 256);
            c->prof->cursor = 0;
            c->prof->capturing = true;
        }
        TJ_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        for (int s = 0; s < group; ++s) issue_step(c);
        TJ_CUDA(c, cudaStreamEndCapture(c->stream, &g));
        TJ_CUDA(c, cudaGraphInstantiate(&c->graph_exec, g, 0));
        cudaGraphDestroy(g);
        if (c->prof) {
            c->prof->capturing = false;
            c->prof->graph_end = c->prof->cursor;
        }
        per_group = c->launches - before;
        c->launches = before;  // counted when launched
        c->graph_steps = group;
        c->graph_launches = per_group;
    }
    per_group = c->graph_launches;
    int remaining = nsteps;
    int n = n0;
    double t = t0;
    while (remaining > 0) {
        bool graph = remaining >= group;
        if (graph) {
            TJ_CUDA(c, cudaGraphLaunch(c->graph_exec, c->stream));
            c->launches += per_group;
            remaining -= group;
        } else {
            for (int s = 0; s < remaining; ++s) issue_step(c);
            remaining = 0;
        }
        e = tj_get_time(c, &t, &n, nullptr);
        if (e) return e;
        if (c->prof) {
            if (graph) c->prof->collect(0, c->prof->graph_end);
            else c->prof->collect_direct();
        }
        DevScalars s;
        TJ_CUDA(c, cudaMemcpyAsync(&s, c->d_scal, sizeof s, cudaMemcpyDeviceToHost, c->stream));
        TJ_CUDA(c, cudaStreamSynchronize(c->stream));
        if (s.done) break;
    }
    if (steps_done) *steps_done = n - n0;
    if (t_out) *t_out = t;
    TJ_CUDA(c, cudaGetLastError());
    return check_status(c);
}

int tj_status(tj_ctx* c)
{
    if (!c) return TJ_ERR_ARG;
    return check_status(c);
}

int tj_synchronize(tj_ctx* c)
{
    if (!c) return TJ_ERR_ARG;
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    return TJ_OK;
}

int tj_launch_count(const tj_ctx* c, long long* count)
{
    if (!c || !count) return TJ_ERR_ARG;
    *count = c->launches;
    return TJ_OK;
}

int tj_get_stream(tj_ctx* c, void** stream)
{
    if (!c || !stream) return TJ_ERR_ARG;
    *stream = (void*)c->stream;
    return TJ_OK;
}

int tj_forward(tj_ctx* c, int q, const double* prim0, const double* eos, int nsteps, const double* dt, int stride)
{
    if (!c || !prim0 || !dt || nsteps < 1 || stride < 1) return fail(c, TJ_ERR_ARG, "bad tj_forward arguments");
    int e = need_state(c);
    if (e) return e;
    if (q != 0) return fail(c, TJ_ERR_ARG, "tj_forward: domain 0 only");
    if (c->params.precision != TJ_PRECISION_FP64) return fail(c, TJ_ERR_ARG, "tj_forward runs the FP64 path");
    // the 2-D fluid adjoint where it applies, the general reverse mode else
    const bool general = adj_unsupported(c->P, (int)c->doms.size()) != nullptr;
    if (general) {
        const char* why = gen_unsupported(c->P, (int)c->doms.size());
        if (why) return fail(c, TJ_ERR_ARG, why);
    }
    for (int n = 0; n < nsteps; ++n)
        if (!(dt[n] > 0.0)) return fail(c, TJ_ERR_ARG, "tj_forward: dt must be positive");
    if (eos)
        for (int m = 0; m < c->P.M; ++m)
            for (int k = 0; k < c->params.materials[m].nparams && k < TJ_MAX_EOS_PARAMS; ++k) {
                c->P.prm[m][k] = eos[m * TJ_MAX_EOS_PARAMS + k];
                c->params.materials[m].params[k] = eos[m * TJ_MAX_EOS_PARAMS + k];
            }
    const DevDomain& D = c->doms[0];
    const size_t nprim = 2 * c->P.M + 4 + (c->P.solid ? 9 : 0) + (c->P.plastic ? c->P.M : 0);
    const size_t bytes = sizeof(double) * nprim * (size_t)c->ntot;
    e = ensure_staging(c, bytes);
    if (e) return e;
    TJ_CUDA(c, cudaMemcpyAsync(c->staging, prim0, bytes, cudaMemcpyDefault, c->stream));
    // a fresh start: THINC scratch zero, as after the reference's allocation
    if (c->ulstar) {
        TJ_CUDA(c, cudaMemsetAsync(c->ulstar, 0, sizeof(double) * c->P.M * c->ntot, c->stream));
        TJ_CUDA(c, cudaMemsetAsync(c->urstar, 0, sizeof(double) * c->P.M * c->ntot, c->stream));
        for (int d = 0; d < 3; ++d)
            if (c->gstar[d])
                TJ_CUDA(c, cudaMemsetAsync(c->gstar[d], 0, sizeof(double) * c->P.M * c->nftot[d], c->stream));
    }
    Fp64Bufs b = bufs(c);
    c->launches += fp64_prim_to_state(c->P, b, 0, c->staging, c->A, c->stream);
    c->adj_general = general;
    long long n;
    if (general) {
        if (!c->gen) c->gen = gen_create();
        n = gen_forward(c->gen, c->P, b, c->staging, (int)nprim, dt, nsteps, stride, c->stream);
    } else {
        if (!c->adj) c->adj = adj_create();
        n = adj_forward(c->adj, c->P, b, D, dt, nsteps, stride, c->stream);
    }
    if (n < 0) return fail(c, (int)n, "tj_forward: device allocation failed");
    c->launches += n;
    TJ_CUDA(c, cudaGetLastError());
    e = check_status(c);
    if (e) return e;
    double t = 0.0;
    for (int k = 0; k < nsteps; ++k) t += dt[k];
    return tj_set_time(c, t, nsteps);
}

int tj_backward(tj_ctx* c, int q, const double* grad_state, double* grad_prim0, double* grad_eos)
{
    if (!c || !grad_state || !grad_prim0 || !grad_eos) return fail(c, TJ_ERR_ARG, "bad tj_backward arguments");
    int e = need_state(c);
    if (e) return e;
    if (q != 0) return fail(c, TJ_ERR_ARG, "tj_backward: domain 0 only");
    if (c->adj_general) {
        if (!c->gen) return fail(c, TJ_ERR_STATE, "tj_backward needs a tj_forward first");
        const long long N = c->ntot;
        const size_t nprim = 2 * c->P.M + 4 + (c->P.solid ? 9 : 0) + (c->P.plastic ? c->P.M : 0);
        const size_t in_w = (size_t)c->P.NCOMP * N, out_w = nprim * (size_t)N;
        e = ensure_staging(c, sizeof(double) * (in_w + out_w));
        if (e) return e;
        double* gin = c->staging;
        double* gout = c->staging + in_w;
        TJ_CUDA(c, cudaMemcpyAsync(gin, grad_state, sizeof(double) * in_w, cudaMemcpyDefault, c->stream));
        int np[TJ_MAX_MATERIALS];
        for (int m = 0; m < c->P.M; ++m) np[m] = c->params.materials[m].nparams;
        Fp64Bufs b = bufs(c);
        long long n = gen_backward(c->gen, c->P, b, gin, gout, grad_eos, np, c->stream);
        if (n < 0) return fail(c, (int)n, "tj_backward: no forward to reverse");
        c->launches += n;
        TJ_CUDA(c, cudaMemcpyAsync(grad_prim0, gout, sizeof(double) * out_w, cudaMemcpyDefault, c->stream));
        TJ_CUDA(c, cudaStreamSynchronize(c->stream));
        TJ_CUDA(c, cudaGetLastError());
        return check_status(c);
    }
    if (!c->adj) return fail(c, TJ_ERR_STATE, "tj_backward needs a tj_forward first");
    const DevDomain& D = c->doms[0];
    const int nx = D.n[0], ny = D.n[1];
    const long long N = c->ntot;
    const size_t in_bytes = sizeof(double) * c->P.NCOMP * (size_t)N;
    const size_t out_bytes = sizeof(double) * (2 * c->P.M + 4) * (size_t)N;
    e = ensure_staging(c, std::max(in_bytes, out_bytes));
    if (e) return e;
    TJ_CUDA(c, cudaMemcpyAsync(c->staging, grad_state, in_bytes, cudaMemcpyDefault, c->stream));
    Fp64Bufs b = bufs(c);
    // the adjoint of the final state in the carried layout, in C (unused by the recompute)
    int bx[6] = {0, 0, 0, nx - 1, ny - 1, 0};
    c->launches += fp64_ap_to_state(c->P, b, 0, bx, c->staging, nx, ny, 1, N, 0, c->C, c->stream);
    long long n = adj_backward(c->adj, c->P, b, D, c->C, c->staging, grad_eos, c->stream);
    if (n < 0) return fail(c, (int)n, "tj_backward: no forward to reverse");
    c->launches += n;
    TJ_CUDA(c, cudaMemcpyAsync(grad_prim0, c->staging, out_bytes, cudaMemcpyDefault, c->stream));
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    TJ_CUDA(c, cudaGetLastError());
    return check_status(c);
}

int tj_tangent(tj_ctx* c, int q, const double* prim0, const double* dprim0, const double* eos, const double* deos,
               int nsteps, const double* dt, double* state, double* dstate)
{
    if (!c || !prim0 || !dt || !dstate || nsteps < 1) return fail(c, TJ_ERR_ARG, "bad tj_tangent arguments");
    int e = need_state(c);
    if (e) return e;
    if (q != 0 || c->doms.size() != 1) return fail(c, TJ_ERR_ARG, "tj_tangent: one domain");
    if (c->params.precision != TJ_PRECISION_FP64) return fail(c, TJ_ERR_ARG, "tj_tangent runs the FP64 path");
    if (c->P.nmix) return fail(c, TJ_ERR_ARG, "tj_tangent: no mixtures (the mixture EOS root find)");
    for (int n = 0; n < nsteps; ++n)
        if (!(dt[n] > 0.0)) return fail(c, TJ_ERR_ARG, "tj_tangent: dt must be positive");
    if (eos)
        for (int m = 0; m < c->P.M; ++m)
            for (int k = 0; k < c->params.materials[m].nparams && k < TJ_MAX_EOS_PARAMS; ++k) {
                c->P.prm[m][k] = eos[m * TJ_MAX_EOS_PARAMS + k];
                c->params.materials[m].params[k] = eos[m * TJ_MAX_EOS_PARAMS + k];
            }
    const size_t N = (size_t)c->ntot;
    const size_t nprim = 2 * c->P.M + 4 + (c->P.solid ? 9 : 0) + (c->P.plastic ? c->P.M : 0);
    const size_t pw = nprim * N, aw = (size_t)c->P.NCOMP * N;
    e = ensure_staging(c, sizeof(double) * (2 * pw + 2 * aw));
    if (e) return e;
    double* prim_dev = c->staging;      // the primitives
    double* dir_dev = prim_dev + pw;    // their direction
    double* ap = dir_dev + pw;          // final values, AccessPattern layout
    double* dap = ap + aw;              // final directions
    TJ_CUDA(c, cudaMemcpyAsync(prim_dev, prim0, sizeof(double) * pw, cudaMemcpyDefault, c->stream));
    if (dprim0) TJ_CUDA(c, cudaMemcpyAsync(dir_dev, dprim0, sizeof(double) * pw, cudaMemcpyDefault, c->stream));
    if (!c->tan) c->tan = tan_create();
    Fp64Bufs b = bufs(c);
    long long n = tan_run(c->tan, c->P, b, 0, prim_dev, dprim0 ? dir_dev : nullptr, deos, nsteps, dt,
                          state ? ap : nullptr, dap, c->stream);
    if (n < 0) return fail(c, (int)n, "tj_tangent: device allocation failed");
    c->launches += n;
    if (state) TJ_CUDA(c, cudaMemcpyAsync(state, ap, sizeof(double) * aw, cudaMemcpyDefault, c->stream));
    TJ_CUDA(c, cudaMemcpyAsync(dstate, dap, sizeof(double) * aw, cudaMemcpyDefault, c->stream));
    int status = 0;
    e = tan_status(c->tan, &status, c->stream);
    if (e) return fail(c, e, "tj_tangent: status read failed");
    TJ_CUDA(c, cudaGetLastError());
    if (status) return fail(c, status, "tj_tangent: a kernel reported an error");
    return TJ_OK;
}

int tj_kernel_config(const tj_ctx* c, char* buf, unsigned long len)
{
    if (!c || !buf || len == 0) return TJ_ERR_ARG;
    if (is_mixed(c)) mixed_describe(c->mixed, buf, len);
    else std::snprintf(buf, len, "fp64 per-direction kernels");
    return TJ_OK;
}

int tj_set_profiling(tj_ctx* c, int on)
{
    if (!c) return TJ_ERR_ARG;
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    if (c->graph_exec) { cudaGraphExecDestroy(c->graph_exec); c->graph_exec = nullptr; }
    if (on && !c->prof) c->prof = new EventProf();
    if (!on && c->prof) { delete c->prof; c->prof = nullptr; }
    return TJ_OK;
}

int tj_kernel_time(tj_ctx* c, const char* kernel, double* ms_total, long long* launches)
{
    if (!c || !kernel) return TJ_ERR_ARG;
    if (ms_total) *ms_total = 0.0;
    if (launches) *launches = 0;
    if (!c->prof) return TJ_OK;
    TJ_CUDA(c, cudaStreamSynchronize(c->stream));
    c->prof->collect_direct();
    for (auto& t : c->prof->totals)
        if (t.first == kernel && ms_total) *ms_total = t.second;
    for (auto& n : c->prof->counts)
        if (n.first == kernel && launches) *launches = n.second;
    return TJ_OK;
}

}  // extern "C"
