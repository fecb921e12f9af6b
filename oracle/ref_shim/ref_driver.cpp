/*
 * ref_driver.cpp -- C entry points around the reference's OWN solver templates, compiled
 * from the PASC_inference sources by oracle/build_ref.sh into oracle/_ref/libpasc_ref.so.
 *
 * TEST INFRASTRUCTURE: it exists to check the FP64 restatement in oracle/pasc_oracle.c
 * against the reference's code and to generate the golden vectors under tests/golden/.
 *
 * Compiled from the reference tree, unmodified:
 *   include/general/solver/spgqpsolver.h   generic SPGQPSolver<VectorBase>::solve/get_fx/compute_dots
 *   include/general/solver/tssolver.h      TSSolver<VectorBase>::solve (outer loop, AIC, annealing)
 *   include/general/solver/{generalsolver,qpsolver,simplesolver,spg_fs}.h
 *   src/general/solver/{generalsolver,spg_fs}.cpp, src/general/{data/generaldata,model/generalmodel}.cpp
 *   include/general/algebra/feasibleset/{generalfeasibleset,simplex_local}.h  (project_sub, sort_bubble)
 *   include/general/data/{qpdata,simpledata,generaldata}.h, include/general/model/{tsmodel,generalmodel}.h
 * Supplied here (the PETSc specialisations cannot be compiled without PETSc):
 *   SimplexFeasibleSet_Local<HostVec>::project   -- the host branch of
 *       src/petscvector/algebra/feasibleset/simplex_local.cpp:52-58 (project_sub per t)
 *   RefH1Model -- the GraphH1FEMModel hooks of src/petscvector/model/graphh1fem.cpp:116-396
 *       restated for the host-array backend (fem not reduced, R = 1).
 */
#include "general/common/common.h"
#include "general/data/qpdata.h"
#include "general/data/simpledata.h"
#include "general/algebra/feasibleset/simplex_local.h"
#include "general/algebra/matrix/blockgraphsparse.h"
#include "general/solver/spgqpsolver.h"
#include "general/solver/simplesolver.h"
#include "general/model/tsmodel.h"
#include "general/solver/tssolver.h"

namespace pascinference {
namespace common {
ConsoleOutput coutMaster;
ConsoleOutput coutAll;
ConsoleArg consoleArg;
GlobalManagerClass GlobalManager;
}
namespace algebra {
std::vector<double> refshim_random_source;
int refshim_nthreads = 1;

/* project_sub works on block t alone (its sort buffer is allocated per call), so the blocks
 * are split over the shim's threads with unchanged results. */
template <>
void SimplexFeasibleSet_Local<HostVec>::project(GeneralVector<HostVec> &x)
{
    double *x_arr = x.arr();
    const int T_ = T, K_ = K;
#pragma omp parallel for schedule(static) num_threads(refshim_nthreads) if (refshim_nthreads > 1)
    for (int t = 0; t < T_; t++) project_sub(x_arr, t, T_, K_);
}
} /* namespace algebra */

namespace model {

/* GraphH1FEMModel hooks for the host-array backend (graphh1fem.cpp, fem not reduced). */
class RefH1Model : public TSModel<HostVec> {
  public:
    QPData<HostVec> *gammadata = NULL;
    SimpleData<HostVec> *thetadata = NULL;
    BlockGraphSparseMatrix<HostVec> *A_shared = NULL;
    double epssqr;
    bool scalef = true;

    RefH1Model(TSData<HostVec> &ts, double epssqr_) : TSModel<HostVec>(ts), epssqr(epssqr_)
    {
        this->thetavectorlength_local = ts.get_K() * ts.get_xdim();
        this->thetavectorlength_global = this->thetavectorlength_local;
        ts.set_model(*this);
    }
    std::string get_name() const { return "Graph-H1-FEM Time-Series Model (host shim)"; }

    double coeffA() const
    {
        double coeff = epssqr; /* graphh1fem.cpp:146-151 */
        if (scalef) coeff *= (1.0 / ((double)this->tsdata->get_T()));
        else coeff *= ((double)this->tsdata->get_T() / ((double)this->tsdata->get_T()));
        return coeff;
    }

    void initialize_gammasolver(GeneralSolver **gammasolver)
    {
        gammadata = new QPData<HostVec>(); /* graphh1fem.cpp:120-182 */
        gammadata->set_x(this->tsdata->get_gammavector());
        gammadata->set_x0(gammadata->get_x());
        gammadata->set_b(new GeneralVector<HostVec>(*gammadata->get_x0()));
        A_shared = new BlockGraphSparseMatrix<HostVec>(*this->tsdata->get_decomposition(), coeffA(), NULL);
        gammadata->set_A(A_shared);
        gammadata->get_x0()->set_random();
        gammadata->set_feasibleset(new SimplexFeasibleSet_Local<HostVec>(
            this->tsdata->get_Tlocal() * this->tsdata->get_Rlocal(), this->tsdata->get_K()));
        *gammasolver = new SPGQPSolver<HostVec>(*gammadata);
    }
    void initialize_thetasolver(GeneralSolver **thetasolver)
    {
        thetadata = new SimpleData<HostVec>();
        thetadata->set_x(this->tsdata->get_thetavector());
        *thetasolver = new SimpleSolver<HostVec>(*thetadata);
    }
    void finalize_gammasolver(GeneralSolver **gammasolver)
    {
        delete *gammasolver;
        *gammasolver = NULL;
    }
    void finalize_thetasolver(GeneralSolver **thetasolver)
    {
        delete *thetasolver;
        *thetasolver = NULL;
    }
    void set_epssqr(double e)
    {
        epssqr = e; /* graphh1fem.h:287-306 */
        if (A_shared) A_shared->set_coeff(coeffA());
    }

    /* graphh1fem.cpp:237-289 */
    void updatebeforesolve_gammasolver(GeneralSolver *)
    {
        int T = this->tsdata->get_T(), K = this->tsdata->get_K(), xdim = this->tsdata->get_xdim();
        const double *theta = this->tsdata->get_thetavector()->arr();
        const double *data = this->tsdata->get_datavector()->arr();
        double *res = gammadata->get_b()->arr();
        for (int t = 0; t < T; t++)
            for (int k = 0; k < K; k++) {
                double r;
                if (xdim == 1) {
                    r = (data[t] - theta[k]) * (data[t] - theta[k]);
                } else {
                    r = 0.0;
                    for (int j = 0; j < xdim; j++) {
                        double dv = data[(size_t)t * xdim + j] - theta[(size_t)k * xdim + j];
                        r += dv * dv;
                    }
                }
                res[(size_t)t * K + k] = r;
            }
        double coeff = -1.0;
        if (scalef) coeff *= (1.0 / ((double)T));
        size_t n = (size_t)T * K;
        for (size_t i = 0; i < n; i++) res[i] = coeff * res[i];
    }

    /* graphh1fem.cpp:306-396 with usethetainpenalty = false */
    void updatebeforesolve_thetasolver(GeneralSolver *)
    {
        int T = this->tsdata->get_T(), K = this->tsdata->get_K(), xdim = this->tsdata->get_xdim();
        const double *gamma = this->tsdata->get_gammavector()->arr();
        const double *data = this->tsdata->get_datavector()->arr();
        double *theta = this->tsdata->get_thetavector()->arr();
        for (int k = 0; k < K; k++) {
            double gsum = 0.0;
            for (int t = 0; t < T; t++) gsum += gamma[(size_t)t * K + k];
            for (int j = 0; j < xdim; j++) {
                double gx = 0.0;
                for (int t = 0; t < T; t++) gx += data[(size_t)t * xdim + j] * gamma[(size_t)t * K + k];
                theta[(size_t)k * xdim + j] = (gsum != 0) ? gx / gsum : 0.0;
            }
        }
    }

    /* graphh1fem.h:368-371 */
    double get_L(GeneralSolver *gammasolver, GeneralSolver *)
    {
        return ((QPSolver<HostVec> *)gammasolver)->get_fx();
    }
    /* graphh1fem.h:444-447 */
    double get_aic(double L) const { return 2 * log(L) + this->tsdata->get_K(); }
};

} /* namespace model */
} /* namespace pascinference */

using namespace pascinference;

/* Exposes TSSolver's iteration counters (protected in the reference class). */
class RefTSSolver : public TSSolver<HostVec> {
  public:
    RefTSSolver(TSData<HostVec> &d, int annealing) : TSSolver<HostVec>(d, annealing) {}
    int it_last_() const { return this->it_last; }
    int it_sum_() const { return this->it_sum; }
};

extern "C" {

void ref_clear_options(void) { consoleArg.overrides.clear(); }
/* Threads of the host-array backend: 1 (or less than 0) every loop and sum sequential in index
 * order; 0 all the threads OpenMP offers, as the oracle's nthreads = 0. */
void ref_set_threads(int n)
{
#ifdef _OPENMP
    if (n == 0) n = omp_get_max_threads();
#endif
    refshim_nthreads = n > 1 ? n : 1;
}
void ref_set_option(const char *name, double value) { consoleArg.overrides[name] = value; }

/* SimplexFeasibleSet_Local<HostVec>::project on T blocks of K doubles, in place. */
int ref_project(double *x, int T, int K)
{
    GeneralVector<HostVec> v((size_t)T * K);
    std::memcpy(v.arr(), x, sizeof(double) * (size_t)T * K);
    SimplexFeasibleSet_Local<HostVec> fs(T, K);
    fs.project(v);
    std::memcpy(x, v.arr(), sizeof(double) * (size_t)T * K);
    return 0;
}

/* SPG_fs (src/general/solver/spg_fs.cpp): init with values[0], then update with values[1..n-1];
 * maxes[i] receives get_max() after step i. */
int ref_fs_sequence(int m, const double *values, int n, double *maxes)
{
    solver::SPG_fs fs(m);
    fs.init(values[0]);
    maxes[0] = fs.get_max();
    for (int i = 1; i < n; i++) {
        fs.update(values[i]);
        maxes[i] = fs.get_max();
    }
    return 0;
}

/* y = coeff * A_hat x with the shim matrix (pins the oracle's stencil to the same assembly). */
int ref_matmult(const double *x, double *y, int T, int K, double coeff)
{
    Decomposition<HostVec> dec(T, 1, K, 1, 1);
    BlockGraphSparseMatrix<HostVec> A(dec, coeff, NULL);
    GeneralVector<HostVec> xv((size_t)T * K), yv((size_t)T * K);
    std::memcpy(xv.arr(), x, sizeof(double) * (size_t)T * K);
    A.matmult(yv, xv);
    std::memcpy(y, yv.arr(), sizeof(double) * (size_t)T * K);
    return 0;
}

/* The reference's generic SPGQPSolver<VectorBase>::solve on one QP.  Settings come from
 * ref_set_option ("spgqpsolver_maxit", ...).  out: it, hessmult, fx. */
int ref_spgqp_solve(const double *b, double *x, int T, int K, double coeff, double *out)
{
    size_t n = (size_t)T * K;
    Decomposition<HostVec> dec(T, 1, K, 1, 1);
    BlockGraphSparseMatrix<HostVec> A(dec, coeff, NULL);
    GeneralVector<HostVec> *xv = new GeneralVector<HostVec>(n);
    GeneralVector<HostVec> *bv = new GeneralVector<HostVec>(n);
    std::memcpy(xv->arr(), x, sizeof(double) * n);
    std::memcpy(bv->arr(), b, sizeof(double) * n);
    QPData<HostVec> qp;
    qp.set_A(&A);
    qp.set_b(bv);
    qp.set_x(xv);
    qp.set_x0(xv);
    SimplexFeasibleSet_Local<HostVec> fs(T, K);
    qp.set_feasibleset(&fs);
    {
        SPGQPSolver<HostVec> solver(qp);
        solver.solve();
        out[0] = solver.get_it();
        out[1] = solver.get_hessmult();
        out[2] = solver.get_fx();
    }
    std::memcpy(x, xv->arr(), sizeof(double) * n);
    delete xv;
    delete bv;
    return 0;
}

/* The reference's TSSolver<VectorBase>::solve with the host-shim FEM-H1 model.
 * gamma_random: what set_random() produces (model initialisation and annealing restarts).
 * theta (K*xdim) in: initial theta (used when "test_theta_given" option is 1); out: final.
 * gamma_out (N): final gamma.  out: L, it_last, it_sum, aic. */
int ref_tssolver_solve(const double *data, const double *gamma_random, double *theta,
                       int T, int K, int xdim, double epssqr, int annealing, int theta_given,
                       double *gamma_out, double *out)
{
    size_t n = (size_t)T * K;
    refshim_random_source.assign(gamma_random, gamma_random + n);
    Decomposition<HostVec> dec(T, 1, K, xdim, 1);
    GeneralVector<HostVec> datav((size_t)T * xdim), gammav(n), thetav((size_t)K * xdim);
    std::memcpy(datav.arr(), data, sizeof(double) * (size_t)T * xdim);
    std::memcpy(thetav.arr(), theta, sizeof(double) * (size_t)K * xdim);
    TSData<HostVec> tsdata(dec, &datav, &gammav, &thetav);
    model::RefH1Model mymodel(tsdata, epssqr);
    {
        RefTSSolver mysolver(tsdata, annealing);
        if (theta_given) mysolver.set_solution_theta(theta);
        mysolver.solve();
        out[0] = mysolver.get_L();
        out[1] = mysolver.it_last_();
        out[2] = mysolver.it_sum_();
        out[3] = tsdata.get_aic();
    }
    std::memcpy(gamma_out, gammav.arr(), sizeof(double) * n);
    std::memcpy(theta, thetav.arr(), sizeof(double) * (size_t)K * xdim);
    refshim_random_source.clear();
    return 0;
}

} /* extern "C" */
