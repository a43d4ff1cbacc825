"""Steady adjoint: the transposed linear solve and the functional derivative
(the reference's linearSolveTranspose, ls_standard.jl:230-244;
evalFunctionalDeriv_q, interface2.jl:259-300; calcAdjoint,
optimization/steady_adjoint.jl:30-89).

The adjoint psi of a functional J at a converged state q solves
(dR/dq)^T psi = -dJ/dq.  With the library's linear solver (an
eulergpu.LinearSolver) the transposed solve is eg_ls_solve_transpose:
GMRES(restart) on J^T M^-T u = b, x = M^-T u, entirely on the device (the
transposed coupling and block-Jacobi applies, device Hessenberg and Givens,
restart cycles replayed as CUDA graphs).  This module orchestrates: it forms
the right-hand side and calls that solve.  For operators of the caller's own
that expose apply_transpose (no library solver), `gmres` below runs the same
Krylov method over those applies with torch vectors.  The functional
derivative is a sum over the boundary faces of one BC group (a few thousand
face nodes), evaluated on the host from the state.
"""
from __future__ import annotations

import math

import numpy as np


class PressureFunctional:
    """The boundary functional of the library: the integral of the pressure
    over the faces of BC group `bc_group` (the reference's
    AbstractFunctional with integratefunctional!, boundary_functional.jl:
    82-126)."""

    def __init__(self, bc_group=0):
        self.bc_group = int(bc_group)


def evalFunctional(mesh, sbp, eqn, opts, functional):
    """J(eqn.q) on the device (eg_calc_functional)."""
    return eqn.gpu.functional_pressure(eqn.q, functional.bc_group)


def evalFunctionalDeriv_q(mesh, sbp, eqn, opts, functional, func_deriv_arr=None, q=None):
    """dJ/dq in the layout of eqn.q: for every boundary face b of the group
    and face node i, with q_f = sum_s interp[f, i, s] q[e, perm[f, s]],
    dJ/dq[e, perm[f, s]] += w_i |n_bi| interp[f, i, s] dp/dq(q_f), where
    p = (gamma - 1)(E - |m|^2 / (2 rho)).  Returns func_deriv_arr (a new
    array when None)."""
    q = np.asarray(eqn.q if q is None else q, dtype=np.float64)
    gamma = float(opts.get("gamma", 1.4))
    g1 = gamma - 1.0
    d = mesh.dim
    out = np.zeros_like(q) if func_deriv_arr is None else func_deriv_arr
    if func_deriv_arr is not None:
        out[...] = 0.0
    lo, hi = int(mesh.bndry_offsets[functional.bc_group]), int(mesh.bndry_offsets[functional.bc_group + 1])
    if hi == lo:
        return out
    e = mesh.bndryfaces[lo:hi, 0]
    f = mesh.bndryfaces[lo:hi, 1]
    perm = sbp.perm[f]                                   # [B, S]
    interp = sbp.interp[f]                               # [B, Nf, S]
    qs = q[e[:, None], perm]                             # [B, S, nv]
    qf = np.einsum("bis,bsc->bic", interp, qs)           # [B, Nf, nv]
    rho = qf[..., 0]
    u = qf[..., 1:d + 1] / rho[..., None]
    dp = np.empty_like(qf)
    dp[..., 0] = 0.5 * g1 * (u * u).sum(axis=-1)
    dp[..., 1:d + 1] = -g1 * u
    dp[..., d + 1] = g1
    wn = sbp.wface[None, :] * np.linalg.norm(mesh.nrm_bndry[lo:hi], axis=-1)   # [B, Nf]
    contrib = np.einsum("bis,bi,bic->bsc", interp, wn, dp)                     # [B, S, nv]
    np.add.at(out, (e[:, None], perm), contrib)
    return out


def _sync(t):
    if t.device.type == "cuda":
        import torch
        torch.cuda.current_stream(t.device).synchronize()


def gmres(apply_op, apply_pc, b, x, restart=30, reltol=1e-10, abstol=0.0, itermax=1000):
    """Solve A x = b by GMRES(restart) with right preconditioning:
    A M u = r0, x = x0 + M u.  apply_op(v, out) / apply_pc(v, out) write
    A v / M v into `out`; b and x are contiguous float64 torch tensors of
    one device (x is the initial guess and is overwritten).  Converged when
    ||b - A x|| <= max(reltol ||b||, abstol).  Returns a dict with iters,
    restarts, converged, res0, res_final (the true residual norm)."""
    import torch
    n = b.numel()
    m = max(1, int(restart))
    dev, dt = b.device, torch.float64
    V = torch.empty((m + 1, n), dtype=dt, device=dev)
    w = torch.empty(n, dtype=dt, device=dev)
    z = torch.empty(n, dtype=dt, device=dev)
    r = torch.empty(n, dtype=dt, device=dev)

    def op(v, out):
        _sync(v)
        apply_op(v, out)

    def pc(v, out):
        _sync(v)
        apply_pc(v, out)

    def residual():
        op(x, r)
        torch.sub(b, r, out=r)
        return float(torch.linalg.vector_norm(r))

    bnorm = float(torch.linalg.vector_norm(b))
    target = max(reltol * bnorm, abstol)
    beta = residual()
    res0, its, restarts = beta, 0, 0
    while beta > target and its < itermax:
        V[0].copy_(r).div_(beta)
        H = np.zeros((m + 1, m))
        cs, sn = np.zeros(m), np.zeros(m)
        g = np.zeros(m + 1)
        g[0] = beta
        k = 0
        for j in range(m):
            pc(V[j], z)
            op(z, w)
            h = V[:j + 1] @ w
            w.sub_(h @ V[:j + 1])
            h2 = V[:j + 1] @ w
            w.sub_(h2 @ V[:j + 1])
            hc = (h + h2).cpu().numpy()
            hn = float(torch.linalg.vector_norm(w))
            H[:j + 1, j] = hc
            H[j + 1, j] = hn
            for i in range(j):
                a, c = H[i, j], H[i + 1, j]
                H[i, j], H[i + 1, j] = cs[i] * a + sn[i] * c, -sn[i] * a + cs[i] * c
            den = math.hypot(H[j, j], H[j + 1, j])
            cs[j], sn[j] = (1.0, 0.0) if den == 0.0 else (H[j, j] / den, H[j + 1, j] / den)
            H[j, j], H[j + 1, j] = den, 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            its += 1
            k = j + 1
            if hn == 0.0 or abs(g[j + 1]) <= target or its >= itermax:
                break
            V[j + 1].copy_(w).div_(hn)
        y = np.zeros(k)
        for i in range(k - 1, -1, -1):
            y[i] = (g[i] - H[i, i + 1:k] @ y[i + 1:k]) / H[i, i]
        u = torch.as_tensor(y, dtype=dt, device=dev) @ V[:k]
        pc(u.contiguous(), z)
        x.add_(z)
        beta = residual()
        restarts += 1
    return {"iters": its, "restarts": max(restarts - 1, 0), "converged": bool(beta <= target),
            "res0": res0, "res_final": beta}


def _as_tensor(a, device):
    import torch
    if isinstance(a, np.ndarray):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).reshape(-1)).to(device)
    return a.reshape(-1)


def linearSolveTranspose(ls, b, x, reltol=None, abstol=None, itermax=None, device=None):
    """x <- solution of J^T x = b with the operator and preconditioner of
    `ls`; b and x are numpy arrays or float64 torch tensors of the mesh's
    size, x the initial guess.  Tolerances default to those set on `ls`
    (set_tolerances), else 1e-10 relative.  An eulergpu.LinearSolver solves
    on the device in the library (eg_ls_solve_transpose; `device` is not
    used); any other object with .lo.apply_transpose, .pc.apply_transpose and
    .restart runs `gmres` with its Krylov vectors on `device` (default: the
    CUDA device when there is one).  Returns the solve's statistics as a dict
    (iters, restarts, converged, res0, res_final)."""
    from . import eulergpu
    if isinstance(ls, eulergpu.LinearSolver):
        if reltol is not None or abstol is not None or itermax is not None:
            ls.set_tolerances(reltol=-1.0 if reltol is None else reltol,
                              abstol=-1.0 if abstol is None else abstol,
                              itermax=-1 if itermax is None else itermax)
        elif ls.reltol is None or ls.reltol <= 0:
            ls.set_tolerances(reltol=1e-10)
        if isinstance(x, np.ndarray):
            xb = np.ascontiguousarray(x, dtype=np.float64).reshape(-1).copy()
            st = ls.solve_transpose(np.ascontiguousarray(b, dtype=np.float64).reshape(-1), xb)
            x[...] = xb.reshape(x.shape)
        else:
            st = ls.solve_transpose(b.reshape(-1).contiguous(), x.reshape(-1))
        return {"iters": st.iters, "restarts": st.restarts, "converged": bool(st.converged),
                "res0": st.res0, "res_final": st.res_final}
    import torch
    if device is None:
        device = ("cuda" if torch.cuda.is_available() else "cpu") if isinstance(b, np.ndarray) else b.device
    rt = getattr(ls, "reltol", -1.0) if reltol is None else reltol
    at = getattr(ls, "abstol", -1.0) if abstol is None else abstol
    im = getattr(ls, "itermax", -1) if itermax is None else itermax
    rt = 1e-10 if rt is None or rt <= 0 else rt
    at = 0.0 if at is None or at < 0 else at
    im = 1000 if im is None or im <= 0 else im
    bt = _as_tensor(b, device).contiguous()
    xt = _as_tensor(x, device).clone().contiguous()
    st = gmres(lambda v, out: ls.lo.apply_transpose(v, out),
               lambda v, out: ls.pc.apply_transpose(v, out),
               bt, xt, restart=getattr(ls, "restart", 30), reltol=rt, abstol=at, itermax=im)
    if isinstance(x, np.ndarray):
        x[...] = xt.cpu().numpy().reshape(x.shape)
    else:
        x.reshape(-1).copy_(xt)
    return st


def evalResidual_revq(mesh, sbp, eqn, opts, res_bar, q_bar, lo=None, zero_output=True):
    """q_bar <- (dR/dq)^T res_bar at eqn.q, or q_bar += it with
    zero_output=False (the reference's reverse-mode residual product,
    interface2.jl:391-430): the explicit Jacobian at eqn.q (into `lo`, a
    LinearOperator of the mesh, or a new FP64 one) applied transposed on the
    device.  res_bar and q_bar are numpy arrays of the state's size.
    Returns q_bar."""
    if lo is None:
        from . import eulergpu
        lo = eulergpu.LinearOperator(eqn.gpu, precision=0)
    lo.calc(eqn.q)
    rb = np.ascontiguousarray(res_bar, dtype=np.float64).reshape(np.shape(eqn.q))
    out = lo.apply_transpose(rb, np.zeros(np.shape(eqn.q))).reshape(np.shape(q_bar))
    if zero_output:
        q_bar[...] = out
    else:
        q_bar += out
    return q_bar


def calcAdjoint(mesh, sbp, eqn, opts, ls, functional, adjoint_vec, recalc_jac=False,
                recalc_pc=False, device=None):
    """adjoint_vec <- psi with (dR/dq)^T psi = -dJ/dq at eqn.q
    (steady_adjoint.jl:30-89).  With recalc_jac / recalc_pc the Jacobian
    and preconditioner of `ls` are first recomputed at eqn.q (the plain
    Jacobian, without the pseudo-time shift of the Newton solve).  `device`
    places the Krylov vectors (see linearSolveTranspose).  Returns the
    transposed solve's statistics."""
    if recalc_jac:
        ls.lo.calc(eqn.q)
    if recalc_pc or recalc_jac:
        ls.pc.calc()
    rhs = -evalFunctionalDeriv_q(mesh, sbp, eqn, opts, functional)
    return linearSolveTranspose(ls, rhs, adjoint_vec, device=device)
