"""Gradient descent on log(epssqr) through the adjoint of the converged gamma step.

The FEM-H1 model has one regularisation weight, epssqr (GraphH1FEMModel(tsdata, epssqr),
include/general/model/graphh1fem.h:75); the reference picks it by sweeping a list of values and
comparing results (examples/test_signal1D/test_signal1D.cpp:268-353).  With a reference signal
at hand (a clean copy, or labels turned into one), the loss
    l(epssqr) = 1/T sum_t (sum_k gamma*_tk(epssqr) theta_k - clean_t)^2
can instead be descended: the gamma step is solved on the GPU, and dl/d epssqr comes from the
adjoint of the converged QP (Problem.recon_mse + Problem.adjoint).  theta is held fixed.
"""
from __future__ import annotations

import math
import time

from . import capi


def descend_log_epssqr(problem, clean, steps: int = 20, lr: float | None = None, first_step: float = 0.5,
                       spg=None, adj=None, min_epssqr: float = 1e-8, polish: bool = True):
    """Runs `steps` gradient steps on u = log(epssqr), starting from problem.epssqr, the
    problem's data, theta and current gamma (each solve warm-starts from the previous gamma).
    lr None: chosen so that the first step moves u by `first_step`.  spg None: each solve runs
    20000 SPG iterations with no stopping test, which brings the mixed path to its fixed point
    on the benchmark sizes (T <= 1e6): the gradient jumps where the free set changes, so it
    has to be taken at the fixed point, not where a |f - f_old| test happened to stop.
    polish: after each solve, Problem.polish moves gamma from the solve's end point (on the
    mixed path an FP32 stall 1e-6..1e-5 from the optimum) onto the optimum of its face.
    Returns one record per step: epssqr, loss, dloss/du, SPG iterations, CG iterations,
    solve and adjoint seconds."""
    spg = spg or capi.spgqp_opts(m=10, maxit=20000, stop_difff=0)
    u = math.log(problem.epssqr)
    out = []
    for step in range(steps + 1):
        eps2 = math.exp(u)
        problem.set_epssqr(eps2)
        problem.update_b()
        t0 = time.perf_counter()
        st = problem.spgqp_solve(spg)
        if polish:
            problem.polish()
        t1 = time.perf_counter()
        loss = problem.recon_mse(clean)
        deps, _, _, ast = problem.adjoint(None, adj)
        t2 = time.perf_counter()
        g = eps2 * deps  # dl/du
        out.append({"epssqr": eps2, "loss": loss, "dloss_dlog_epssqr": g, "spg_it": st.it,
                    "cg_it": ast.cg_it, "solve_s": t1 - t0, "adjoint_s": t2 - t1})
        if step == steps:
            break
        if lr is None:
            lr = first_step / abs(g) if g != 0.0 else 0.0
        u = max(u - lr * g, math.log(min_epssqr))
    return out
