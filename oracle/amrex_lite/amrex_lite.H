// amrex_lite: a project-written stand-in for the small part of AMReX that the
// Tenjin per-timestep update touches. TEST INFRASTRUCTURE ONLY: it exists so
// that the reference's own hot-path sources can be compiled unchanged into the
// oracle under oracle/_ref. Nothing in the product links it.
//
// AMReX itself is not vendored by the reference (Make.package lists sources
// only), so its version is unpinned. This header restates the documented
// semantics of the calls the reference makes:
//   * FArrayBox / Array4: component-major SoA, i fastest, then j, k, n
//     (boxaccesscellarray.cpp:19-65 indexes fab.array()(i,j,k,n)).
//   * MultiFab::Copy / Add / mult: element-wise over valid + nghost cells
//     (cellarray.cpp:80-99).
//   * MultiFab::min(comp): minimum over valid cells (timestep.cpp:63).
//   * FillBoundary: ghost cells that lie inside the domain take the value of
//     the box whose valid region holds them (hllc.cpp:645-646,691).
//   * FillDomainBoundary: ghost cells outside the domain are mapped back into
//     the domain one direction at a time (foextrap: nearest boundary cell;
//     reflect_even / reflect_odd: mirror image, negated for odd), and read
//     from the valid data (main.cpp:124, hllc.cpp:642-643, boundary.cpp:3-42).
//     AMReX's filcc reads a corner ghost through the fab's own not-yet-filled
//     interior ghost; this shim reads the valid owner instead. The two differ
//     only at a physical-boundary corner next to an interior box boundary.
//   * BoxArray::maxSize: AMReX's BoxList::maxSize chop (powers of two
//     factored out, near-equal pieces, chopped from the high end).
//   * MFIter: box order; inside an OpenMP parallel region each thread takes a
//     contiguous block of boxes.
// IntVect always stores three integers with the unused ones zero; the
// reference reads extra[z] of a 2-D IntVect at hllc.cpp:148,397.
#ifndef AMREX_LITE_H
#define AMREX_LITE_H

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <sstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

// The reference names std::__cxx11::string (simulationheader.h:34), which
// GCC 13's libstdc++ no longer declares under that name.
namespace std { inline namespace __cxx11 { using string = ::std::basic_string<char>; } }

#ifndef AMREX_SPACEDIM
#error "AMREX_SPACEDIM must be defined (1, 2 or 3)"
#endif

#if AMREX_SPACEDIM == 1
#define AMREX_D_DECL(a, b, c) a
#elif AMREX_SPACEDIM == 2
#define AMREX_D_DECL(a, b, c) a, b
#else
#define AMREX_D_DECL(a, b, c) a, b, c
#endif

namespace amrex {

using Real = double;

template <class T>
using Vector = std::vector<T>;

template <class T, std::size_t N>
using Array = std::array<T, N>;

inline std::ostream& Print() { return std::cout; }

// AllPrintToFile(name) << ...: the text is collected in a string stream with
// the stream's default precision (6 significant digits) and appended to the
// file when the statement ends. AMReX's own class is version-dependent (some
// versions suffix the file name with the rank); one serial process here
// appends to the name as given.
class PrintToFile {
public:
    explicit PrintToFile(std::string name) : name_(std::move(name)) {}
    ~PrintToFile()
    {
        std::ofstream f(name_, std::ios_base::app);
        f << ss_.str();
    }
    template <class T>
    PrintToFile& operator<<(const T& v)
    {
        ss_ << v;
        return *this;
    }
    PrintToFile& operator<<(std::ostream& (*m)(std::ostream&))
    {
        ss_ << m;
        return *this;
    }

private:
    std::string name_;
    std::ostringstream ss_;
};

using AllPrintToFile = PrintToFile;

inline double second()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

inline std::string Concatenate(const std::string& root, int num, int mindigits = 5)
{
    std::string s = std::to_string(num);
    while ((int)s.size() < mindigits) s = "0" + s;
    return root + s;
}

struct Dim3 {
    int x, y, z;
};

class IntVect {
public:
    IntVect(int a = 0, int b = 0, int c = 0) : v{a, b, c} {}
    int& operator[](int i) { return v[i]; }
    const int& operator[](int i) const { return v[i]; }
    int v[3];
};

class Box {
public:
    Box() : lo(0, 0, 0), hi(-1, -1, -1) {}
    Box(const IntVect& l, const IntVect& h) : lo(l), hi(h)
    {
        for (int d = AMREX_SPACEDIM; d < 3; ++d) { lo[d] = 0; hi[d] = 0; }
    }
    const IntVect& smallEnd() const { return lo; }
    const IntVect& bigEnd() const { return hi; }
    int length(int d) const { return hi[d] - lo[d] + 1; }
    long numPts() const
    {
        long n = 1;
        for (int d = 0; d < 3; ++d) n *= (long)length(d);
        return n;
    }
    bool contains(int i, int j, int k) const
    {
        return i >= lo[0] && i <= hi[0] && j >= lo[1] && j <= hi[1] && k >= lo[2] && k <= hi[2];
    }
    Box grow(int ng) const
    {
        Box b = *this;
        for (int d = 0; d < AMREX_SPACEDIM; ++d) { b.lo[d] -= ng; b.hi[d] += ng; }
        return b;
    }
    // Chop at pos along dir: *this keeps [lo, pos-1], the returned box is [pos, hi].
    Box chop(int dir, int pos)
    {
        Box upper = *this;
        upper.lo[dir] = pos;
        hi[dir] = pos - 1;
        return upper;
    }
    IntVect lo, hi;
};

inline Dim3 lbound(const Box& b) { return Dim3{b.lo[0], b.lo[1], b.lo[2]}; }
inline Dim3 ubound(const Box& b) { return Dim3{b.hi[0], b.hi[1], b.hi[2]}; }

template <class T>
struct Array4 {
    T* p;
    Dim3 begin;
    long jstride, kstride, nstride;
    T& operator()(int i, int j, int k, int n) const
    {
        return p[(i - begin.x) + (long)(j - begin.y) * jstride + (long)(k - begin.z) * kstride + (long)n * nstride];
    }
};

template <class T>
class BaseFab {
public:
    BaseFab() : ncomp(0) {}
    void define(const Box& b, int nc)
    {
        box = b;
        ncomp = nc;
        data.assign((size_t)b.numPts() * nc, T(0));  // zero-initialised
    }
    Array4<T> array()
    {
        Array4<T> a;
        a.p = data.data();
        a.begin = lbound(box);
        a.jstride = box.length(0);
        a.kstride = (long)box.length(0) * box.length(1);
        a.nstride = box.numPts();
        return a;
    }
    T& at(int i, int j, int k, int n) { return array()(i, j, k, n); }
    Box box;  // allocated (grown) box
    int ncomp;
    std::vector<T> data;
};

using FArrayBox = BaseFab<Real>;
using IArrayBox = BaseFab<int>;

class BoxArray {
public:
    BoxArray() {}
    explicit BoxArray(const Box& b) : boxes{b} {}
    int size() const { return (int)boxes.size(); }
    const Box& operator[](int i) const { return boxes[i]; }
    void maxSize(int chunk)
    {
        for (int dir = 0; dir < AMREX_SPACEDIM; ++dir) {
            std::vector<Box> out;
            for (Box bx : boxes) {
                int len = bx.length(dir);
                if (len > chunk) {
                    int ratio = 1, bs = chunk, nlen = len;
                    while ((bs % 2 == 0) && (nlen % 2 == 0)) { ratio *= 2; bs /= 2; nlen /= 2; }
                    int numblk = nlen / bs + (nlen % bs ? 1 : 0);
                    int sz = nlen / numblk, ex = nlen % numblk;
                    for (int k = 0; k < numblk - 1; ++k) {
                        int ksize = (k < ex) ? sz + 1 : sz;
                        int pos = bx.hi[dir] - ksize * ratio + 1;
                        out.push_back(bx.chop(dir, pos));
                    }
                }
                out.push_back(bx);
            }
            boxes.swap(out);
        }
    }
    void surroundingNodes(int dir)
    {
        nodal_dir = dir;
        for (auto& b : boxes) b.hi[dir] += 1;
    }
    std::vector<Box> boxes;
    int nodal_dir = -1;
};

class DistributionMapping {
public:
    DistributionMapping() {}
    explicit DistributionMapping(const BoxArray&) {}
};

struct Periodicity {};

class RealBox {
public:
    RealBox() {}
    RealBox(std::initializer_list<Real> l, std::initializer_list<Real> h)
    {
        int d = 0;
        for (Real v : l) lo[d++] = v;
        d = 0;
        for (Real v : h) hi[d++] = v;
    }
    Real lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
};

namespace CoordSys { enum CoordType { cartesian = 0 }; }

class Geometry {
public:
    Geometry() {}
    Geometry(const Box& dom, const RealBox& rb, int, std::initializer_list<int>) : domain(dom), rbox(rb)
    {
        for (int d = 0; d < 3; ++d) dxv[d] = (rb.hi[d] - rb.lo[d]) / (Real)dom.length(d);
    }
    const Box& Domain() const { return domain; }
    const Real* CellSize() const { return dxv; }
    Periodicity periodicity() const { return Periodicity{}; }
    Box domain;
    RealBox rbox;
    Real dxv[3] = {1, 1, 1};
};

namespace BCType {
enum mathematicalBndryTypes { bogus = -666, reflect_odd = -1, int_dir = 0, reflect_even = 1, foextrap = 2, ext_dir = 3, hoextrap = 4 };
}

class BCRec {
public:
    BCRec() : lo{BCType::foextrap, BCType::foextrap, BCType::foextrap}, hi{BCType::foextrap, BCType::foextrap, BCType::foextrap} {}
    void setLo(int dir, int t) { lo[dir] = t; }
    void setHi(int dir, int t) { hi[dir] = t; }
    int lo[3], hi[3];
};

template <class T>
class FabArray;

class MFIter {
public:
    template <class FA>
    explicit MFIter(const FA& fa) : ba(&fa.boxArray())
    {
        int n = ba->size();
        beginIndex = 0;
        endIndex = n;
#ifdef _OPENMP
        if (omp_in_parallel()) {
            int nt = omp_get_num_threads(), tid = omp_get_thread_num();
            beginIndex = (int)((long)n * tid / nt);
            endIndex = (int)((long)n * (tid + 1) / nt);
        }
#endif
        idx = beginIndex;
    }
    bool isValid() const { return idx < endIndex; }
    void operator++() { ++idx; }
    int index() const { return idx; }
    const Box& validbox() const { return ba->boxes[idx]; }
    const BoxArray* ba;
    int idx, beginIndex, endIndex;
};

template <class T>
class FabArray {
public:
    FabArray() {}
    FabArray(const BoxArray& b, const DistributionMapping& dm, int nc, int ng) { define(b, dm, nc, ng); }
    void define(const BoxArray& b, const DistributionMapping&, int nc, int ng)
    {
        ba = b;
        ncomp = nc;
        ngrow = ng;
        fabs.assign(ba.size(), BaseFab<T>());
        for (int i = 0; i < ba.size(); ++i) fabs[i].define(ba[i].grow(ng), nc);
    }
    const BoxArray& boxArray() const { return ba; }
    int nComp() const { return ncomp; }
    int nGrow() const { return ngrow; }
    BaseFab<T>& operator[](const MFIter& mfi) { return fabs[mfi.index()]; }
    BaseFab<T>& operator[](int i) { return fabs[i]; }

    // Owner of a cell inside the domain: the box whose valid region holds it.
    // A lookup table over the bounding box of the valid boxes, built once.
    int owner(int i, int j, int k)
    {
        if (owner_tab.empty()) {
            for (int d = 0; d < 3; ++d) { olo[d] = ba[0].lo[d]; ohi[d] = ba[0].hi[d]; }
            for (int b = 0; b < ba.size(); ++b)
                for (int d = 0; d < 3; ++d) { olo[d] = std::min(olo[d], ba[b].lo[d]); ohi[d] = std::max(ohi[d], ba[b].hi[d]); }
            long n = 1;
            for (int d = 0; d < 3; ++d) n *= (long)(ohi[d] - olo[d] + 1);
            owner_tab.assign(n, -1);
            for (int b = 0; b < ba.size(); ++b) {
                const Box& vb = ba[b];
                for (int kk = vb.lo[2]; kk <= vb.hi[2]; ++kk)
                    for (int jj = vb.lo[1]; jj <= vb.hi[1]; ++jj)
                        for (int ii = vb.lo[0]; ii <= vb.hi[0]; ++ii) owner_tab[otab(ii, jj, kk)] = b;
            }
        }
        if (i < olo[0] || i > ohi[0] || j < olo[1] || j > ohi[1] || k < olo[2] || k > ohi[2]) return -1;
        return owner_tab[otab(i, j, k)];
    }
    long otab(int i, int j, int k) const
    {
        return (i - olo[0]) + (long)(ohi[0] - olo[0] + 1) * ((j - olo[1]) + (long)(ohi[1] - olo[1] + 1) * (k - olo[2]));
    }
    std::vector<int> owner_tab;
    int olo[3], ohi[3];

    // Ghost cells inside the domain take the owner's valid value.
    void FillBoundary(const Periodicity& = Periodicity{})
    {
        for (int b = 0; b < ba.size(); ++b) {
            const Box& vb = ba[b];
            Box gb = vb.grow(ngrow);
            for (int o = 0; o < ba.size(); ++o) {
                if (o == b) continue;
                const Box& ob = ba[o];
                int lo[3], hi[3];
                bool empty = false;
                for (int d = 0; d < 3; ++d) {
                    lo[d] = std::max(gb.lo[d], ob.lo[d]);
                    hi[d] = std::min(gb.hi[d], ob.hi[d]);
                    if (lo[d] > hi[d]) empty = true;
                }
                if (empty) continue;
                auto dst = fabs[b].array();
                auto src = fabs[o].array();
                for (int n = 0; n < ncomp; ++n)
                    for (int k = lo[2]; k <= hi[2]; ++k)
                        for (int j = lo[1]; j <= hi[1]; ++j)
                            for (int i = lo[0]; i <= hi[0]; ++i) dst(i, j, k, n) = src(i, j, k, n);
            }
        }
    }

    BoxArray ba;
    int ncomp = 0, ngrow = 0;
    std::vector<BaseFab<T>> fabs;
};

class MultiFab : public FabArray<Real> {
public:
    MultiFab() {}
    MultiFab(const BoxArray& b, const DistributionMapping& dm, int nc, int ng) : FabArray<Real>(b, dm, nc, ng) {}

    static void Copy(MultiFab& dst, const MultiFab& src, int srccomp, int dstcomp, int nc, int ng)
    {
        for (int b = 0; b < dst.ba.size(); ++b) {
            auto d = dst.fabs[b].array();
            auto s = const_cast<MultiFab&>(src).fabs[b].array();
            Box gb = dst.ba[b].grow(ng);
            for (int n = 0; n < nc; ++n)
                for (int k = gb.lo[2]; k <= gb.hi[2]; ++k)
                    for (int j = gb.lo[1]; j <= gb.hi[1]; ++j)
                        for (int i = gb.lo[0]; i <= gb.hi[0]; ++i) d(i, j, k, dstcomp + n) = s(i, j, k, srccomp + n);
        }
    }
    static void Add(MultiFab& dst, const MultiFab& src, int srccomp, int dstcomp, int nc, int ng)
    {
        for (int b = 0; b < dst.ba.size(); ++b) {
            auto d = dst.fabs[b].array();
            auto s = const_cast<MultiFab&>(src).fabs[b].array();
            Box gb = dst.ba[b].grow(ng);
            for (int n = 0; n < nc; ++n)
                for (int k = gb.lo[2]; k <= gb.hi[2]; ++k)
                    for (int j = gb.lo[1]; j <= gb.hi[1]; ++j)
                        for (int i = gb.lo[0]; i <= gb.hi[0]; ++i) d(i, j, k, dstcomp + n) += s(i, j, k, srccomp + n);
        }
    }
    void mult(Real v, int comp, int nc, int ng)
    {
        for (int b = 0; b < ba.size(); ++b) {
            auto d = fabs[b].array();
            Box gb = ba[b].grow(ng);
            for (int n = 0; n < nc; ++n)
                for (int k = gb.lo[2]; k <= gb.hi[2]; ++k)
                    for (int j = gb.lo[1]; j <= gb.hi[1]; ++j)
                        for (int i = gb.lo[0]; i <= gb.hi[0]; ++i) d(i, j, k, comp + n) *= v;
        }
    }
    Real min(int comp, int = 0, bool = false) const
    {
        Real m = std::numeric_limits<Real>::max();
        for (int b = 0; b < ba.size(); ++b) {
            auto d = const_cast<MultiFab*>(this)->fabs[b].array();
            const Box& vb = ba[b];
            for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
                for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
                    for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) m = std::min(m, d(i, j, k, comp));
        }
        return m;
    }
};

class iMultiFab : public FabArray<int> {
public:
    iMultiFab() {}
    iMultiFab(const BoxArray& b, const DistributionMapping& dm, int nc, int ng) : FabArray<int>(b, dm, nc, ng) {}
};

// Physical-boundary ghost fill (see the header comment for the semantics).
inline void FillDomainBoundary(MultiFab& mf, const Geometry& geom, const Vector<BCRec>& bc)
{
    const Box& dom = geom.Domain();
    for (int b = 0; b < mf.ba.size(); ++b) {
        Box gb = mf.ba[b].grow(mf.ngrow);
        auto dst = mf.fabs[b].array();
        for (int k = gb.lo[2]; k <= gb.hi[2]; ++k)
            for (int j = gb.lo[1]; j <= gb.hi[1]; ++j)
                for (int i = gb.lo[0]; i <= gb.hi[0]; ++i) {
                    int idx[3] = {i, j, k};
                    bool outside = false;
                    for (int d = 0; d < AMREX_SPACEDIM; ++d)
                        if (idx[d] < dom.lo[d] || idx[d] > dom.hi[d]) outside = true;
                    if (!outside) continue;
                    for (int n = 0; n < mf.ncomp; ++n) {
                        int m[3] = {i, j, k};
                        Real sign = 1.0;
                        for (int d = 0; d < AMREX_SPACEDIM; ++d) {
                            if (m[d] < dom.lo[d]) {
                                int t = bc[n].lo[d];
                                if (t == BCType::reflect_even || t == BCType::reflect_odd) {
                                    m[d] = 2 * dom.lo[d] - 1 - m[d];
                                    if (t == BCType::reflect_odd) sign = -sign;
                                } else {
                                    m[d] = dom.lo[d];
                                }
                            } else if (m[d] > dom.hi[d]) {
                                int t = bc[n].hi[d];
                                if (t == BCType::reflect_even || t == BCType::reflect_odd) {
                                    m[d] = 2 * dom.hi[d] + 1 - m[d];
                                    if (t == BCType::reflect_odd) sign = -sign;
                                } else {
                                    m[d] = dom.hi[d];
                                }
                            }
                        }
                        int o = mf.owner(m[0], m[1], m[2]);
                        Real v = mf.fabs[o].array()(m[0], m[1], m[2], n);
                        dst(i, j, k, n) = (sign < 0.0) ? -v : v;
                    }
                }
    }
}

inline void Initialize(int, char**) {}
inline void Finalize() {}

}  // namespace amrex

#endif
