/*
 * Shim for the reference's TSData over the host-array backend (oracle/build_ref.sh only;
 * test infrastructure): the getters TSSolver and TSModel use, nothing else.
 */
#ifndef PASC_REFSHIM_TSDATA_H
#define PASC_REFSHIM_TSDATA_H

#include "general/common/common.h"
#include "general/data/generaldata.h"

namespace pascinference {
namespace model { template <class VectorBase> class TSModel; }
namespace data {

template <class VectorBase> class TSData : public GeneralData {
  public:
    Decomposition<VectorBase> *decomposition;
    GeneralVector<VectorBase> *datavector, *gammavector, *thetavector;
    model::TSModel<VectorBase> *tsmodel;
    double aic_solution;

    TSData(Decomposition<VectorBase> &dec, GeneralVector<VectorBase> *data,
           GeneralVector<VectorBase> *gamma, GeneralVector<VectorBase> *theta)
        : decomposition(&dec), datavector(data), gammavector(gamma), thetavector(theta),
          tsmodel(NULL), aic_solution(std::numeric_limits<double>::max()) {}
    std::string get_name() const { return "TSData"; }
    void set_model(model::TSModel<VectorBase> &m) { tsmodel = &m; }
    model::TSModel<VectorBase> *get_model() const { return tsmodel; }
    Decomposition<VectorBase> *get_decomposition() const { return decomposition; }
    GeneralVector<VectorBase> *get_datavector() const { return datavector; }
    GeneralVector<VectorBase> *get_gammavector() const { return gammavector; }
    GeneralVector<VectorBase> *get_thetavector() const { return thetavector; }
    int get_T() const { return decomposition->get_T(); }
    int get_Tlocal() const { return decomposition->get_Tlocal(); }
    int get_R() const { return decomposition->get_R(); }
    int get_Rlocal() const { return decomposition->get_Rlocal(); }
    int get_K() const { return decomposition->get_K(); }
    int get_xdim() const { return decomposition->get_xdim(); }
    double get_aic() const { return aic_solution; }
    void set_aic(double a) { aic_solution = a; }
};

} /* namespace data */
} /* namespace pascinference */
#endif
