/*
 * Shim for the reference's BlockGraphSparseMatrix over the host-array backend
 * (oracle/build_ref.sh only; test infrastructure).  matmult restates the assembled matrix of
 * src/petscvector/algebra/matrix/blockgraphsparse.cpp:51-109 for R = 1 (diagonal 2 at the
 * ends, 4 inside, 0 for T == 1; -2 at t-1 and t+1), multiplied row by row over ascending
 * columns from 0.0 like a CSR MatMult, then scaled by alpha (:152-188, coeffs == NULL).
 * Rows are independent, so refshim_nthreads threads give the same values as one.
 */
#ifndef PASC_REFSHIM_BLOCKGRAPHSPARSE_H
#define PASC_REFSHIM_BLOCKGRAPHSPARSE_H

#include "general/common/common.h"

namespace pascinference {
namespace algebra {

template <class VectorBase> class BlockGraphSparseMatrix : public GeneralMatrix<VectorBase> {
    Decomposition<VectorBase> *decomposition;
    double alpha;
  public:
    BlockGraphSparseMatrix(Decomposition<VectorBase> &dec, double alpha_ = 1.0,
                           GeneralVector<VectorBase> * /*coeffs*/ = NULL)
        : decomposition(&dec), alpha(alpha_) {}
    std::string get_name() const { return "BlockGraphSparseMatrix"; }
    double get_coeff() const { return alpha; }
    void set_coeff(double c) { alpha = c; }
    int get_T() const { return decomposition->get_T(); }
    int get_K() const { return decomposition->get_K(); }
    void matmult(VectorBase &y, const VectorBase &x) const {
        long T = decomposition->get_T();
        int K = decomposition->get_K();
        const double *xa = x.arr();
        double *ya = y.arr();
        long n = T * (long)K;
#pragma omp parallel for schedule(static) num_threads(refshim_nthreads) if (refshim_nthreads > 1)
        for (long i = 0; i < n; i++) {
            long t = i / K;
            double sum = 0.0;
            if (T == 1) {
                sum += 0.0 * xa[i];
            } else {
                double wsum = (t == 0 || t == T - 1) ? 2.0 : 4.0;
                if (t > 0) sum += -2.0 * xa[i - K];
                sum += wsum * xa[i];
                if (t < T - 1) sum += -2.0 * xa[i + K];
            }
            ya[i] = sum;
        }
#pragma omp parallel for schedule(static) num_threads(refshim_nthreads) if (refshim_nthreads > 1)
        for (long i = 0; i < n; i++) ya[i] = alpha * ya[i];
    }
};

} /* namespace algebra */
} /* namespace pascinference */
#endif
