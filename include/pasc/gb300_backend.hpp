// gb300_backend.hpp -- a GB300 backend for PASC_inference's own generic solver templates.
//
// The reference's solvers are templates over a vector type; a backend is a vector type plus
// explicit specialisations of the classes whose generic bodies are empty (the PETSc backend's
// are declared in include/external/petscvector/solver/spgqpsolver.h:20-34 and
// include/external/petscvector/algebra/matrix/blockgraphsparse.h:15-25).  This header is that
// backend for a GB300: GB300Vec keeps its values in FP64 device memory, and
//   GeneralVector<GB300Vec>                      = copy, = x - a*g, = x - y, = A*x, -= y,
//                                                 += a*x, dot, norm, set_random
//                                                 (include/general/algebra/vector/generalvector.h:58-106)
//   BlockGraphSparseMatrix<GB300Vec>::matmult     pasc_gb300_fem_h1_matmult_f64
//                                                 (src/petscvector/algebra/matrix/blockgraphsparse.cpp:152-160)
//   SimplexFeasibleSet_Local<GB300Vec>::project   pasc_gb300_project_f64
//                                                 (src/petscvector/algebra/feasibleset/simplex_local.cpp:38-65)
//   GB300H1FEMModel                               the GraphH1FEMModel hooks on the device: residual b
//                                                 and the theta step (src/petscvector/model/graphh1fem.cpp:
//                                                 116-396, fem not reduced, one rank)
// so that the reference's SPGQPSolver<GB300Vec>::solve (include/general/solver/spgqpsolver.h:
// 575-805) and TSSolver<GB300Vec>::solve (include/general/solver/tssolver.h:492-715) run
// unchanged with every vector operation on the GPU: FP64, one C-ABI call per operation of the
// reference (the fused FP32 sweep of pasc_gb300_spgqp_solve is the other, faster route).
//
// Include it after the reference's headers that declare the primary templates it
// specialises (general/algebra/vector/generalvector.h, general/algebra/matrix/
// blockgraphsparse.h, general/algebra/feasibleset/simplex_local.h, general/data/qpdata.h,
// general/data/simpledata.h, general/data/tsdata.h, general/model/tsmodel.h,
// general/solver/spgqpsolver.h, general/solver/simplesolver.h), and link libpasc_gb300.so.
//
// The generic TSSolver permutes gamma and sets a given theta through the PETSc Vec of a vector
// (get_vector(), tssolver.h:760-790), which a device vector does not have: run it with
// tssolver_init_permute = 0 after permuting gamma with GB300Vec::permute_blocked, and set theta
// through the theta vector (GB300Vec::upload).  get_vector() throws to say so.
#pragma once

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "pasc_gb300.h"

namespace pascinference {
namespace algebra {

inline void gb300_check(int rc)
{
    if (rc != PASC_OK) throw std::runtime_error(std::string("pasc_gb300: ") + pasc_gb300_last_error());
}

// The vector type of the backend: n FP64 values on one device, owned.
class GB300Vec {
public:
    GB300Vec() {}
    explicit GB300Vec(long n, int device = 0) : n_(n), device_(device) { gb300_check(pasc_gb300_vec_alloc(&d_, n, device)); }
    // "new GeneralVector(*pattern)": same size and device as the pattern (zeroed)
    GB300Vec(const GB300Vec &pattern) : n_(pattern.n_), device_(pattern.device_)
    {
        if (n_ > 0 || pattern.d_) gb300_check(pasc_gb300_vec_alloc(&d_, n_, device_));
    }
    GB300Vec &operator=(const GB300Vec &) = delete;
    ~GB300Vec()
    {
        if (d_) pasc_gb300_vec_free(d_);
    }
    double *dev() { return d_; }
    const double *dev() const { return d_; }
    long size() const { return n_; }
    int local_size() const { return (int)n_; }
    int device() const { return device_; }
    void upload(const std::vector<double> &v) { gb300_check(pasc_gb300_vec_set(d_, v.data(), n_)); }
    std::vector<double> download() const
    {
        std::vector<double> v((size_t)n_);
        gb300_check(pasc_gb300_vec_get(d_, v.data(), n_));
        return v;
    }
    // Decomposition::permute_TRK (src/petscvector/common/decomposition.cpp:266-356, R = 1):
    // blocked k*T + t -> interleaved t*K + k, in place through a temporary
    void permute_blocked(long T, int K)
    {
        GB300Vec tmp(*this);
        gb300_check(pasc_gb300_permute_f64(d_, tmp.d_, T, K, nullptr));
        gb300_check(pasc_gb300_vec_copy(d_, tmp.d_, n_, nullptr));
    }

protected:
    double *d_ = nullptr;
    long n_ = 0;
    int device_ = 0;
};

// What set_random() produces, installed by the caller (the reference draws it with PETSc's
// generator, src/petscvector/algebra/vector/generalvector.cpp:7-28).
inline std::vector<double> &gb300_random_source()
{
    static std::vector<double> v;
    return v;
}

template <>
class GeneralVector<GB300Vec> : public GB300Vec {
public:
    struct Scaled {
        double a;
        const GeneralVector *x;
    };
    struct DiffScaled {
        const GeneralVector *x;
        Scaled s;
    };
    struct Diff {
        const GeneralVector *x, *y;
    };
    struct MatVec {
        const GeneralMatrix<GB300Vec> *A;
        const GeneralVector *x;
    };

    GeneralVector() : GB300Vec() {}
    explicit GeneralVector(long n, int device = 0) : GB300Vec(n, device) {}
    GeneralVector(const GeneralVector &pattern) : GB300Vec(pattern) {}

    static std::string get_name() { return "GB300Vec"; }

    GeneralVector &operator=(const GeneralVector &o)
    {
        if (this != &o) gb300_check(pasc_gb300_vec_copy(d_, o.d_, n_, nullptr));
        return *this;
    }
    GeneralVector &operator=(const DiffScaled &e)  // x - a*g  (VecWAXPY)
    {
        gb300_check(pasc_gb300_vec_waxpy(d_, -e.s.a, e.s.x->d_, e.x->d_, n_, nullptr));
        return *this;
    }
    GeneralVector &operator=(const Diff &e)  // x - y
    {
        gb300_check(pasc_gb300_vec_waxpy(d_, -1.0, e.y->d_, e.x->d_, n_, nullptr));
        return *this;
    }
    GeneralVector &operator=(const MatVec &e);
    GeneralVector &operator-=(const GeneralVector &o)
    {
        gb300_check(pasc_gb300_vec_axpy(d_, -1.0, o.d_, n_, nullptr));
        return *this;
    }
    GeneralVector &operator+=(const Scaled &s)
    {
        gb300_check(pasc_gb300_vec_axpy(d_, s.a, s.x->d_, n_, nullptr));
        return *this;
    }
    void set_random()
    {
        const std::vector<double> &src = gb300_random_source();
        if ((long)src.size() == n_) upload(src);
    }
    void valuesUpdate() {}
    // the PETSc Vec the generic TSSolver reaches for (see the header comment)
    [[noreturn]] Vec get_vector() const
    {
        throw std::runtime_error("GB300Vec has no PETSc Vec: permute with permute_blocked and run TSSolver with "
                                 "tssolver_init_permute = 0; set theta through the theta vector");
    }
};

inline GeneralVector<GB300Vec>::Scaled operator*(double a, const GeneralVector<GB300Vec> &x) { return {a, &x}; }
inline GeneralVector<GB300Vec>::DiffScaled operator-(const GeneralVector<GB300Vec> &x,
                                                     const GeneralVector<GB300Vec>::Scaled &s)
{
    return {&x, s};
}
inline GeneralVector<GB300Vec>::Diff operator-(const GeneralVector<GB300Vec> &x, const GeneralVector<GB300Vec> &y)
{
    return {&x, &y};
}
inline GeneralVector<GB300Vec>::MatVec operator*(const GeneralMatrix<GB300Vec> &A, const GeneralVector<GB300Vec> &x)
{
    return {&A, &x};
}
inline GeneralVector<GB300Vec> &GeneralVector<GB300Vec>::operator=(const MatVec &e)
{
    e.A->matmult(*this, *e.x);
    return *this;
}

inline double dot(const GeneralVector<GB300Vec> &a, const GeneralVector<GB300Vec> &b)
{
    double s = 0.0;
    gb300_check(pasc_gb300_vec_dot(a.dev(), b.dev(), a.size(), &s, nullptr));
    return s;
}
inline double norm(const GeneralVector<GB300Vec> &a) { return std::sqrt(dot(a, a)); }
inline double sum(const GeneralVector<GB300Vec> &a)
{
    GeneralVector<GB300Vec> one(a);
    std::vector<double> ones((size_t)a.size(), 1.0);
    one.upload(ones);
    return dot(a, one);
}
template <class Stream>
inline Stream &operator<<(Stream &o, const GeneralVector<GB300Vec> &)
{
    return o;
}

// y = coeff * A_hat x on the device (the assembled FEM-H1 row, MatMult of blockgraphsparse.cpp:
// 152-160 for R = 1, without theta coefficients)
template <>
inline void BlockGraphSparseMatrix<GB300Vec>::matmult(GB300Vec &y, const GB300Vec &x) const
{
    gb300_check(pasc_gb300_fem_h1_matmult_f64(x.dev(), y.dev(), this->get_T(), this->get_K(), this->get_coeff(),
                                              nullptr));
}

// projection of every timestep's K values onto the simplex, on the device, in the reference's
// operation order (simplex_local.cu:70-139)
template <>
inline void SimplexFeasibleSet_Local<GB300Vec>::project(GeneralVector<GB300Vec> &x)
{
    gb300_check(pasc_gb300_project_f64(x.dev(), this->T, this->K, nullptr));
}

}  // namespace algebra

namespace model {

// The GraphH1FEMModel hooks for device vectors (fem not reduced, one rank, scalar data,
// usethetainpenalty = false): A = epssqr/T * A_hat, b = -(x_t - theta_k)^2 / T
// (graphh1fem.cpp:116-214, 237-289), theta_k = sum_t gamma_tk x_t / sum_t gamma_tk (:347-380),
// L = the gamma solver's objective (include/general/model/graphh1fem.h:368-371), AIC = 2 log L
// + K (:444-447).  The gamma QP's x is the TSData gamma vector itself (graphh1fem.cpp:136).
class GB300H1FEMModel : public TSModel<algebra::GB300Vec> {
    using V = algebra::GB300Vec;

public:
    GB300H1FEMModel(TSData<V> &ts, double epssqr) : TSModel<V>(ts), epssqr_(epssqr)
    {
        this->thetavectorlength_local = ts.get_K() * ts.get_xdim();
        this->thetavectorlength_global = this->thetavectorlength_local;
        ts.set_model(*this);
    }
    std::string get_name() const { return "Graph-H1-FEM Time-Series Model (GB300 device vectors)"; }
    double coeffA() const { return epssqr_ * (1.0 / (double)this->tsdata->get_T()); }

    void initialize_gammasolver(GeneralSolver **gammasolver)
    {
        gammadata_ = new QPData<V>();
        gammadata_->set_x(this->tsdata->get_gammavector());
        gammadata_->set_x0(gammadata_->get_x());
        b_ = new algebra::GeneralVector<V>(*gammadata_->get_x0());
        gammadata_->set_b(b_);
        A_ = new BlockGraphSparseMatrix<V>(*this->tsdata->get_decomposition(), coeffA(), NULL);
        gammadata_->set_A(A_);
        fs_ = new SimplexFeasibleSet_Local<V>(this->tsdata->get_Tlocal() * this->tsdata->get_Rlocal(),
                                              this->tsdata->get_K());
        gammadata_->set_feasibleset(fs_);
        *gammasolver = new SPGQPSolver<V>(*gammadata_);
    }
    void initialize_thetasolver(GeneralSolver **thetasolver)
    {
        thetadata_ = new SimpleData<V>();
        thetadata_->set_x(this->tsdata->get_thetavector());
        *thetasolver = new SimpleSolver<V>(*thetadata_);
    }
    void finalize_gammasolver(GeneralSolver **gammasolver)
    {
        delete *gammasolver;
        *gammasolver = NULL;
        delete fs_;
        delete A_;
        delete b_;
        delete gammadata_;
        fs_ = NULL;
        A_ = NULL;
        b_ = NULL;
        gammadata_ = NULL;
    }
    void finalize_thetasolver(GeneralSolver **thetasolver)
    {
        delete *thetasolver;
        *thetasolver = NULL;
        delete thetadata_;
        thetadata_ = NULL;
    }
    void set_epssqr(double e)
    {
        epssqr_ = e;
        if (A_) A_->set_coeff(coeffA());
    }
    void updatebeforesolve_gammasolver(GeneralSolver *)
    {
        const long T = this->tsdata->get_T();
        algebra::gb300_check(pasc_gb300_residual_f64(this->tsdata->get_datavector()->dev(),
                                                     this->tsdata->get_thetavector()->dev(), b_->dev(), T,
                                                     this->tsdata->get_K(), -1.0 * (1.0 / (double)T), nullptr));
    }
    void updatebeforesolve_thetasolver(GeneralSolver *)
    {
        algebra::gb300_check(pasc_gb300_theta_update_f64(this->tsdata->get_gammavector()->dev(),
                                                         this->tsdata->get_datavector()->dev(),
                                                         this->tsdata->get_thetavector()->dev(),
                                                         this->tsdata->get_T(), this->tsdata->get_K(), nullptr));
    }
    double get_L(GeneralSolver *gammasolver, GeneralSolver *) { return ((QPSolver<V> *)gammasolver)->get_fx(); }
    double get_aic(double L) const { return 2 * log(L) + this->tsdata->get_K(); }

private:
    double epssqr_;
    QPData<V> *gammadata_ = NULL;
    SimpleData<V> *thetadata_ = NULL;
    algebra::GeneralVector<V> *b_ = NULL;
    BlockGraphSparseMatrix<V> *A_ = NULL;
    SimplexFeasibleSet_Local<V> *fs_ = NULL;
};

}  // namespace model
}  // namespace pascinference
