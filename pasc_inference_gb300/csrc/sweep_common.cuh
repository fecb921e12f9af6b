// sweep_common.cuh -- the scalar part of an SPG sweep, shared by the sweep kernels: the last
// block of the grid turns the reduced sums (w[0] = sum (g-b)'x, w[1] = d'd, w[2] = sum of
// squared neighbour differences of d, w[3] = g'd) into the reference's step-length, GLL and
// stopping decisions (src/petscvector/solver/spgqpsolver.cpp:131-274, src/general/solver/
// spg_fs.cpp), in FP64, and writes the scalars of the next sweep.  With st->coeffmode the rules
// are SPGQPSolverC's (include/general/solver/spgqpsolver_coeff.h:611-835): d'Ad without the
// coefficient eps, BB step einv*dd/dAd, A-condition with 2*eps*xi and the sigma1 clamp applied
// to beta_hat itself; the sweeps take alpha and beta in the usual units either way.
#pragma once

#include "common.cuh"
#include "internal.h"

namespace pasc {

template <bool INIT>
__device__ __forceinline__ void spg_finish_sweep(SpgDevState *st, int cur, const double (&w)[4])
{
    st->counter = 0;
    st->sweeps += 1;
    const double fnew = 0.5 * w[0];
    const double dd = w[1];
    const bool cm = st->coeffmode != 0;
    const double eps = st->coeff, einv = eps == 0.0 ? 1.0 : 1.0 / eps;
    const double dAd = cm ? 2.0 * w[2] : 2.0 * st->coeff * w[2];  // the solver's own d'Ad
    const double gd = w[3];

    if (INIT) {
        // spgqpsolver.cpp:131-137: fs.init(fx), fx_old = max
        st->fx = fnew;
        st->fx_old = DBL_MAX;
        for (int q = 0; q < st->m; q++) st->fs[q] = fnew;
        st->fs_last = 0;
        st->it = 0;
        st->hessmult = 1;
        st->cur = cur ^ 1;
        if (st->maxit <= 0) { st->status = PASC_SPG_MAXIT; return; }
        if (!isfinite(fnew)) { st->status = PASC_SPG_NONFINITE; return; }
    } else {
        st->it += 1;
        st->hessmult += 1;
        st->cur = cur ^ 1;
        st->fx_old = st->fx;  // :207
        st->fx = fnew;        // :209
        int li = st->fs_last + 1;  // fs.update, spg_fs.cpp:52-63
        if (li >= st->m) li = 0;
        st->fs[li] = fnew;
        st->fs_last = li;
        if (!isfinite(fnew)) { st->status = PASC_SPG_NONFINITE; return; }
        // stopping tests of iteration it on the direction it applied (:260-274).  f - f_old
        // is taken in the incremental form f(x + beta d) - f(x) = beta g'd + beta^2 d'Ad / 2
        // (SPGQPSolver::get_fx(fx_old, beta, gd, dAd), include/general/solver/
        // spgqpsolver.h:809-842): equal in exact arithmetic, and free of the cancellation of
        // two objectives summed from FP32 terms (their difference is resolved only to ~1e-7
        // of f, far above the usual eps, so the explicit form would stop on rounding noise)
        const double ddo = st->dd, dAdo = st->dAd;
        const double dAdtrue = cm ? eps * dAdo : dAdo;
        const double dfx = st->beta * st->gd + 0.5 * st->beta * st->beta * dAdtrue;
        if ((st->stop_difff && fabs(dfx) < st->eps) ||
            (st->stop_normgp && ddo < st->eps) ||
            (st->stop_normgp_normb && ddo < st->eps * st->normb) ||
            (st->stop_Anormgp && dAdo < st->eps) ||
            (st->stop_Anormgp_normb && dAdo < st->eps * st->normb)) {
            st->status = PASC_SPG_CONVERGED;
            return;
        }
        if (st->it >= st->maxit) { st->status = PASC_SPG_MAXIT; return; }
    }

    // next direction: step length from the A-condition (:176-195) and BB step (:216)
    if (!(isfinite(dd) && isfinite(dAd) && isfinite(gd))) { st->status = PASC_SPG_NONFINITE; return; }
    if (!(dd > 0.0)) { st->status = PASC_SPG_DAD_ZERO; return; }  // projected step vanished
    double nbeta, nalpha;
    if (dAd > 0.0) {
        double fx_max = st->fs[0];
        for (int q = 0; q < st->m; q++) fx_max = st->fs[q] > fx_max ? st->fs[q] : fx_max;
        const double xi = (fx_max - st->fx) / dAd;
        const double beta_bar = -gd / dAd;
        if (cm) {
            double beta_hat = st->gamma * beta_bar + sqrt(st->gamma * st->gamma * beta_bar * beta_bar + 2 * eps * xi);
            if (einv * beta_hat < st->sigma1) beta_hat = st->sigma1;
            nbeta = einv * beta_hat < st->sigma2 ? einv * beta_hat : st->sigma2;
            nalpha = einv * (dd / dAd);
        } else {
            double beta_hat = st->gamma * beta_bar + sqrt(st->gamma * st->gamma * beta_bar * beta_bar + 2 * xi);
            if (beta_hat < st->sigma1) beta_hat = st->sigma1;
            nbeta = beta_hat < st->sigma2 ? beta_hat : st->sigma2;
            nalpha = dd / dAd;
        }
    } else if (gd < 0.0) {
        // d'Ad = 0 with d != 0: the objective is linear along d (A_hat d = 0, e.g. T == 1).
        // The reference divides by zero here; its comparisons then fall through to
        // beta = sigma2.  Take that step and keep the step length finite.
        nbeta = st->sigma2;
        nalpha = st->alpha_cur;
    } else {
        st->status = PASC_SPG_DAD_ZERO;
        return;
    }
    st->alpha_prev = st->alpha_cur;
    st->alpha_cur = nalpha;
    st->beta = nbeta;
    st->dd = dd;
    st->dAd = dAd;
    st->gd = gd;
}

}  // namespace pasc
