/*
 * Shim for the reference's Decomposition (oracle/build_ref.sh only; test infrastructure).
 * One rank, R = 1: the layout helpers the generic solver templates call.  permute_TRK
 * restates src/petscvector/common/decomposition.cpp:266-356 for that case:
 * new[t*K + k] = orig[k*T + t] (invert copies the other way).
 */
#ifndef PASC_REFSHIM_DECOMPOSITION_H
#define PASC_REFSHIM_DECOMPOSITION_H

#include "general/common/common.h"

namespace pascinference {
namespace common {

template <class VectorBase> class Decomposition {
    int T, R, K, xdim;
  public:
    Decomposition(int T_, int R_, int K_, int xdim_, int /*DDT_size*/) : T(T_), R(R_), K(K_), xdim(xdim_) {}
    int get_T() const { return T; }
    int get_Tlocal() const { return T; }
    int get_Tbegin() const { return 0; }
    int get_Tend() const { return T; }
    int get_R() const { return R; }
    int get_Rlocal() const { return R; }
    int get_K() const { return K; }
    int get_xdim() const { return xdim; }
    void print(ConsoleOutput &) const {}
    void permute_TRK(Vec orig, Vec nw, bool invert = false) const {
        for (int k = 0; k < K; k++)
            for (int t = 0; t < T; t++) {
                if (!invert) nw->v[(size_t)t * K + k] = orig->v[(size_t)k * T + t];
                else orig->v[(size_t)k * T + t] = nw->v[(size_t)t * K + k];
            }
    }
};

} /* namespace common */
} /* namespace pascinference */
#endif
