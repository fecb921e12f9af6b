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

// Order-preserving integer key of a finite double (larger value, larger key), and back: the
// GLL maximum is taken on integer compares, which do not wait on the FP64 pipe.
__device__ __forceinline__ long long fs_key(double x)
{
    const long long b = __double_as_longlong(x);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double fs_unkey(long long k) { return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL)); }

// h: the state as the sweep found it (read only; a snapshot in shared memory where the caller
// has one, else *st itself); the new state is written to *st.  The reads of h and the writes
// to st are independent, so a snapshot turns the ~20 dependent round trips to global memory of
// the step logic into shared-memory loads (at T = 1e7, K = 3 the step logic with the state read
// in place took 4.5 us of the 56.8 us sweep).
template <bool INIT>
__device__ __forceinline__ void spg_finish_sweep(SpgDevState *st, const SpgDevState &h, int cur, const double (&w)[4])
{
    st->counter = 0;
    st->sweeps = h.sweeps + 1;
    const double fnew = 0.5 * w[0];
    const double dd = w[1];
    const bool cm = h.coeffmode != 0;
    const double eps = h.coeff;
    const double dAd = cm ? 2.0 * w[2] : 2.0 * eps * w[2];  // the solver's own d'Ad
    const double gd = w[3];
    const int m = h.m;
    int li = 0;  // the GLL slot that now holds fnew (INIT: all of them)

    if (INIT) {
        // spgqpsolver.cpp:131-137: fs.init(fx), fx_old = max
        st->fx = fnew;
        st->fx_old = DBL_MAX;
        for (int q = 0; q < m; q++) st->fs[q] = fnew;
        st->fs_last = 0;
        st->it = 0;
        st->hessmult = 1;
        st->cur = cur ^ 1;
        if (h.maxit <= 0) { st->status = PASC_SPG_MAXIT; return; }
        if (!isfinite(fnew)) { st->status = PASC_SPG_NONFINITE; return; }
    } else {
        const int it1 = h.it + 1;  // (h may be *st itself: read before the writes below)
        st->it = it1;
        st->hessmult = h.hessmult + 1;
        st->cur = cur ^ 1;
        st->fx_old = h.fx;  // :207
        st->fx = fnew;      // :209
        li = h.fs_last + 1;  // fs.update, spg_fs.cpp:52-63
        if (li >= m) li = 0;
        st->fs[li] = fnew;
        st->fs_last = li;
        if (!isfinite(fnew)) { st->status = PASC_SPG_NONFINITE; return; }
        // stopping tests of iteration it on the direction it applied (:260-274).  f - f_old
        // is taken in the incremental form f(x + beta d) - f(x) = beta g'd + beta^2 d'Ad / 2
        // (SPGQPSolver::get_fx(fx_old, beta, gd, dAd), include/general/solver/
        // spgqpsolver.h:809-842): equal in exact arithmetic, and free of the cancellation of
        // two objectives summed from FP32 terms (their difference is resolved only to ~1e-7
        // of f, far above the usual eps, so the explicit form would stop on rounding noise)
        const double ddo = h.dd, dAdo = h.dAd;
        const double dAdtrue = cm ? eps * dAdo : dAdo;
        const double dfx = h.beta * h.gd + 0.5 * h.beta * h.beta * dAdtrue;
        if ((h.stop_difff && fabs(dfx) < h.eps) ||
            (h.stop_normgp && ddo < h.eps) ||
            (h.stop_normgp_normb && ddo < h.eps * h.normb) ||
            (h.stop_Anormgp && dAdo < h.eps) ||
            (h.stop_Anormgp_normb && dAdo < h.eps * h.normb)) {
            st->status = PASC_SPG_CONVERGED;
            return;
        }
        if (it1 >= h.maxit) { st->status = PASC_SPG_MAXIT; return; }
    }

    // next direction: step length from the A-condition (:176-195) and BB step (:216)
    if (!(isfinite(dd) && isfinite(dAd) && isfinite(gd))) { st->status = PASC_SPG_NONFINITE; return; }
    if (!(dd > 0.0)) { st->status = PASC_SPG_DAD_ZERO; return; }  // projected step vanished
    double nbeta, nalpha;
    if (dAd > 0.0) {
        // max of the GLL ring (its values are finite: a non-finite f ends the solve above)
        long long k0 = fs_key(fnew), k1 = k0;
        if (!INIT) {
            int q = 0;
            for (; q + 1 < m; q += 2) {
                const long long a = fs_key(q == li ? fnew : h.fs[q]), b = fs_key(q + 1 == li ? fnew : h.fs[q + 1]);
                k0 = a > k0 ? a : k0;
                k1 = b > k1 ? b : k1;
            }
            if (q < m) {
                const long long a = fs_key(q == li ? fnew : h.fs[q]);
                k0 = a > k0 ? a : k0;
            }
        }
        const double fx_max = fs_unkey(k0 > k1 ? k0 : k1);
        const double dxi = fx_max - fnew;  // >= 0, in FP64 (a difference of close objectives)
        // The step lengths go to the sweeps as FP32; their rules (xi, beta_bar, the A-condition
        // root, the BB ratio) run in FP32 on operands scaled by the power of two 2^-e that
        // brings d'Ad to [1, 2) (exact, and the three ratios do not change), which keeps the
        // FP32 range out of the way; a d'Ad outside 2^-120..2^120 takes the FP64 path.
        const long long bits = __double_as_longlong(dAd);
        const int e = (int)((bits >> 52) & 0x7ff) - 1023;
        if (e > -120 && e < 120) {
            const double sc = __longlong_as_double((long long)(1023 - e) << 52);
            const float a = (float)(dAd * sc), fdx = (float)(dxi * sc), fgd = (float)(-gd * sc), fdd = (float)(dd * sc);
            const float xi = fdx / a, beta_bar = fgd / a, g = (float)h.gamma;
            if (cm) {
                const float epsf = (float)eps, einv = eps == 0.0 ? 1.f : 1.f / epsf;
                float beta_hat = g * beta_bar + sqrtf(g * g * beta_bar * beta_bar + 2.f * epsf * xi);
                double bh = (double)(einv * beta_hat);
                if (bh < h.sigma1) beta_hat = (float)h.sigma1, bh = h.sigma1;
                bh = (double)(einv * beta_hat);
                nbeta = bh < h.sigma2 ? bh : h.sigma2;
                nalpha = (double)(einv * (fdd / a));
            } else {
                const float beta_hat = g * beta_bar + sqrtf(g * g * beta_bar * beta_bar + 2.f * xi);
                double bh = (double)beta_hat;
                if (bh < h.sigma1) bh = h.sigma1;
                nbeta = bh < h.sigma2 ? bh : h.sigma2;
                nalpha = (double)(fdd / a);
            }
        } else {
            const double xi = dxi / dAd;
            const double beta_bar = -gd / dAd;
            if (cm) {
                const double einv = eps == 0.0 ? 1.0 : 1.0 / eps;
                double beta_hat = h.gamma * beta_bar + sqrt(h.gamma * h.gamma * beta_bar * beta_bar + 2 * eps * xi);
                if (einv * beta_hat < h.sigma1) beta_hat = h.sigma1;
                nbeta = einv * beta_hat < h.sigma2 ? einv * beta_hat : h.sigma2;
                nalpha = einv * (dd / dAd);
            } else {
                double beta_hat = h.gamma * beta_bar + sqrt(h.gamma * h.gamma * beta_bar * beta_bar + 2 * xi);
                if (beta_hat < h.sigma1) beta_hat = h.sigma1;
                nbeta = beta_hat < h.sigma2 ? beta_hat : h.sigma2;
                nalpha = dd / dAd;
            }
        }
    } else if (gd < 0.0) {
        // d'Ad = 0 with d != 0: the objective is linear along d (A_hat d = 0, e.g. T == 1).
        // The reference divides by zero here; its comparisons then fall through to
        // beta = sigma2.  Take that step and keep the step length finite.
        nbeta = h.sigma2;
        nalpha = h.alpha_cur;
    } else {
        st->status = PASC_SPG_DAD_ZERO;
        return;
    }
    st->alpha_prev = h.alpha_cur;
    st->alpha_cur = nalpha;
    st->beta = nbeta;
    st->dd = dd;
    st->dAd = dAd;
    st->gd = gd;
}

// The state read in place (kernels without room for a snapshot).
template <bool INIT>
__device__ __forceinline__ void spg_finish_sweep(SpgDevState *st, int cur, const double (&w)[4])
{
    spg_finish_sweep<INIT>(st, *st, cur, w);
}

}  // namespace pasc
