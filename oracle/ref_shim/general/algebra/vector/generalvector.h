/*
 * Shim for the reference's GeneralVector / GeneralMatrix over a plain host array backend
 * (oracle/build_ref.sh only; test infrastructure).
 *
 * The expression forms the reference's generic SPGQPSolver / TSSolver bodies use are
 * evaluated element by element in the obvious order:
 *   d = x - a*g   ->  d_i = x_i - a*g_i        d -= x   ->  d_i = d_i - x_i
 *   x += a*d      ->  x_i = x_i + a*d_i        t = g - b ->  t_i = g_i - b_i
 *   y = A*x       ->  A.matmult(y, x)          dot(a,b) ->  sequential sum of a_i*b_i
 *
 * refshim_nthreads (default 1) splits the element-wise loops over OpenMP threads; dot() then
 * sums static chunks [n*id/cnt, n*(id+1)/cnt) and the chunk sums in thread order -- the scheme
 * of the oracle's multi-threaded mode, so the two give the same bits at the same thread count.
 * With 1 thread every loop and sum runs sequentially in index order, as above.
 */
#ifndef PASC_REFSHIM_GENERALVECTOR_H
#define PASC_REFSHIM_GENERALVECTOR_H

#include "general/common/common.h"
#ifdef _OPENMP
#include <omp.h>
#endif

namespace pascinference {
namespace algebra {

/* The VectorBase of this backend: owns a host array reachable as a PETSc-like Vec. */
class HostVec {
  public:
    Vec h;
    HostVec() : h(new RefShimVec()) {}
    explicit HostVec(size_t n) : h(new RefShimVec()) { h->v.assign(n, 0.0); }
    HostVec(const HostVec &o) : h(new RefShimVec()) { h->v.assign(o.h->v.size(), 0.0); }
    ~HostVec() { delete h; }
    HostVec &operator=(const HostVec &) = delete;
    Vec get_vector() const { return h; }
    double *arr() { return h->v.data(); }
    const double *arr() const { return h->v.data(); }
    int size() const { return (int)h->v.size(); }
    int local_size() const { return (int)h->v.size(); }
};

template <class VectorBase> class GeneralVector;
template <class VectorBase> class GeneralMatrix;

/* Random source for set_random(): the driver installs the vector it wants produced. */
extern std::vector<double> refshim_random_source;
/* Threads of the loops below (set by ref_set_threads). */
extern int refshim_nthreads;

template <> class GeneralVector<HostVec> : public HostVec {
  public:
    struct Scaled { double a; const GeneralVector *x; };
    struct DiffScaled { const GeneralVector *x; Scaled s; };
    struct Diff { const GeneralVector *x; const GeneralVector *y; };
    struct MatVec { const GeneralMatrix<HostVec> *A; const GeneralVector *x; };

    GeneralVector() : HostVec() {}
    explicit GeneralVector(size_t n) : HostVec(n) {}
    /* "new GeneralVector(*pattern)": same layout as the pattern (values are set before use) */
    GeneralVector(const GeneralVector &pattern) : HostVec(pattern) {}

    static std::string get_name() { return "HostVec"; }

    GeneralVector &operator=(const GeneralVector &o) {
        if (this != &o) h->v = o.h->v;
        return *this;
    }
    GeneralVector &operator=(const DiffScaled &e) {
        const long n = (long)h->v.size();
        double *y = h->v.data();
        const double *a = e.x->h->v.data(), *g = e.s.x->h->v.data();
        const double c = e.s.a;
#pragma omp parallel for schedule(static) num_threads(refshim_nthreads) if (refshim_nthreads > 1)
        for (long i = 0; i < n; i++) y[i] = a[i] - c * g[i];
        return *this;
    }
    GeneralVector &operator=(const Diff &e) {
        const long n = (long)h->v.size();
        double *y = h->v.data();
        const double *a = e.x->h->v.data(), *b = e.y->h->v.data();
#pragma omp parallel for schedule(static) num_threads(refshim_nthreads) if (refshim_nthreads > 1)
        for (long i = 0; i < n; i++) y[i] = a[i] - b[i];
        return *this;
    }
    GeneralVector &operator=(const MatVec &e);
    GeneralVector &operator-=(const GeneralVector &o) {
        const long n = (long)h->v.size();
        double *y = h->v.data();
        const double *a = o.h->v.data();
#pragma omp parallel for schedule(static) num_threads(refshim_nthreads) if (refshim_nthreads > 1)
        for (long i = 0; i < n; i++) y[i] = y[i] - a[i];
        return *this;
    }
    GeneralVector &operator+=(const Scaled &s) {
        const long n = (long)h->v.size();
        double *y = h->v.data();
        const double *a = s.x->h->v.data();
        const double c = s.a;
#pragma omp parallel for schedule(static) num_threads(refshim_nthreads) if (refshim_nthreads > 1)
        for (long i = 0; i < n; i++) y[i] = y[i] + c * a[i];
        return *this;
    }
    void set_random() {
        if (refshim_random_source.size() == h->v.size()) h->v = refshim_random_source;
    }
    void valuesUpdate() {}
};

inline GeneralVector<HostVec>::Scaled operator*(double a, const GeneralVector<HostVec> &x) { return {a, &x}; }
inline GeneralVector<HostVec>::DiffScaled operator-(const GeneralVector<HostVec> &x,
                                                    const GeneralVector<HostVec>::Scaled &s) { return {&x, s}; }
inline GeneralVector<HostVec>::Diff operator-(const GeneralVector<HostVec> &x,
                                              const GeneralVector<HostVec> &y) { return {&x, &y}; }

inline double dot(const GeneralVector<HostVec> &a, const GeneralVector<HostVec> &b) {
    const double *x = a.h->v.data(), *y = b.h->v.data();
    const long n = (long)a.h->v.size();
    if (refshim_nthreads <= 1) {
        double s = 0.0;
        for (long i = 0; i < n; i++) s += x[i] * y[i];
        return s;
    }
    double part[256];
    const int nt = refshim_nthreads > 256 ? 256 : refshim_nthreads;
    int used = 1;
#pragma omp parallel num_threads(nt)
    {
        int id = 0, cnt = 1;
#ifdef _OPENMP
        id = omp_get_thread_num();
        cnt = omp_get_num_threads();
#endif
        const long lo = n * id / cnt, hi = n * (id + 1) / cnt;
        double s = 0.0;
        for (long i = lo; i < hi; i++) s += x[i] * y[i];
        part[id] = s;
        if (id == 0) used = cnt;
    }
    double tot = 0.0;
    for (int j = 0; j < used; j++) tot += part[j];
    return tot;
}
inline double norm(const GeneralVector<HostVec> &a) { return std::sqrt(dot(a, a)); }
inline std::ostream &operator<<(std::ostream &o, const GeneralVector<HostVec> &) { return o; }

template <class VectorBase> class GeneralMatrix {
  public:
    virtual ~GeneralMatrix() {}
    virtual void print(ConsoleOutput &) const {}
    virtual void print(ConsoleOutput &, ConsoleOutput &) const {}
    virtual void printcontent(ConsoleOutput &) const {}
    virtual std::string get_name() const { return "GeneralMatrix"; }
    virtual void matmult(VectorBase &y, const VectorBase &x) const = 0;
};

inline GeneralVector<HostVec>::MatVec operator*(const GeneralMatrix<HostVec> &A, const GeneralVector<HostVec> &x) {
    return {&A, &x};
}
inline GeneralVector<HostVec> &GeneralVector<HostVec>::operator=(const MatVec &e) {
    e.A->matmult(*this, *e.x);
    return *this;
}

} /* namespace algebra */
} /* namespace pascinference */
#endif
