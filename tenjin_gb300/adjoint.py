"""Gradients of the FP64 per-timestep update through the adjoint pair
``tj_forward`` / ``tj_backward`` of libtenjin_gpu.so, behind the
``torch.autograd.Function`` contract.

The reference has no adjoint. What is differentiated is its FP64 update
(advance and the post-advance operators, main.cpp:145-187, hllc.cpp:579-707)
over a time-step schedule frozen from a plain FP64 run at the reference
parameters (the dt of timestep.cpp:36-70 and main.cpp:128-143): 2-D fluids
with the stiffened-gas EOS by the dedicated reverse sweep, every other
configuration without BVD-THINC and mixtures (solids, plasticity, 1-D, 3-D)
by the general reverse mode. Inputs are the initial primitive fields (the
layout ``tj_set_primitive`` takes: alpha[M], rho_k[M], u[3], p, V[9] for
solids, epsilon[M] with plasticity) and the raw EOS parameter vectors
(``getMaterialParameters`` order, initialise.cpp:125-235); the output is the
final state in the AccessPattern layout. ``AdjointRun.tangent`` gives the
forward-mode derivative of the same run along a direction.

    run = AdjointRun(case)
    dts = run.dt_schedule(200)
    state = TenjinRun.apply(prim0, eos, run, dts, 20)   # checkpoint every 20 steps
    J = objective(state); J.backward()                   # prim0.grad, eos.grad

Gradients with respect to (gamma, p_inf) follow from ``eos_vector`` by torch's
own chain rule (p_ref = -gamma p_inf).
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np
import torch

from . import _lib
from .cases import Case
from .host import FP64, TenjinGPU

MAX_EOS = _lib.TJ_MAX_EOS_PARAMS


def _ptr(t: torch.Tensor) -> ctypes.c_void_p:
    assert t.is_contiguous() and t.dtype == torch.float64
    return ctypes.c_void_p(t.data_ptr())


class AdjointRun:
    """An FP64 context for forward/backward and tangent passes over one domain."""

    def __init__(self, case: Case):
        self.case = case
        self.sim = TenjinGPU(case, FP64, set_initial=False)
        d = case.domains[0]
        self.shape_state = (self.sim.ncomp, d.n_cells[2], d.n_cells[1], d.n_cells[0])
        self.shape_prim = (case.nprim, d.n_cells[2], d.n_cells[1], d.n_cells[0])
        self.M = case.M
        self._ready = False

    def dt_schedule(self, nsteps: int, prim0: Optional[np.ndarray] = None) -> np.ndarray:
        """dt of each step of a plain FP64 run (getTimeStep with the reference's
        clamps) from the case's initial state, in a context of its own."""
        ref = TenjinGPU(self.case, FP64, set_initial=False)
        ref.set_primitive(0, self.case.domains[0].prim if prim0 is None else prim0)
        dts = np.empty(nsteps)
        for n in range(nsteps):
            ref.step()
            dts[n] = ref.time()[2]
        ref.close()
        return dts

    def eos_array(self) -> np.ndarray:
        e = np.zeros((self.M, MAX_EOS))
        for m, mat in enumerate(self.case.materials):
            e[m, :len(mat.params)] = mat.params
        return e

    def forward(self, prim0: torch.Tensor, eos: np.ndarray, dts: np.ndarray, stride: int,
                out: Optional[torch.Tensor] = None) -> torch.Tensor:
        prim0 = prim0.detach().contiguous().to(torch.float64)
        eos = np.ascontiguousarray(eos, dtype=np.float64)
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        if prim0.is_cuda:
            torch.cuda.current_stream().synchronize()
        L = self.sim.L
        self.sim._check(L.tj_forward(self.sim.h, 0, _ptr(prim0), eos.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     len(dts), dts.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(stride)))
        self._ready = True
        if out is None:
            out = torch.empty(self.shape_state, dtype=torch.float64, device=prim0.device)
        self.sim._check(L.tj_download_domain(self.sim.h, 0, ctypes.cast(_ptr(out), ctypes.POINTER(ctypes.c_double))))
        return out

    def backward(self, grad_state: torch.Tensor, grad_prim: Optional[torch.Tensor] = None):
        if not self._ready:
            raise RuntimeError("backward needs a forward first")
        g = grad_state.detach().contiguous().to(torch.float64)
        if g.is_cuda:
            torch.cuda.current_stream().synchronize()
        if grad_prim is None:
            grad_prim = torch.empty(self.shape_prim, dtype=torch.float64, device=g.device)
        ge = np.zeros((self.M, MAX_EOS))
        self.sim._check(self.sim.L.tj_backward(self.sim.h, 0, _ptr(g), _ptr(grad_prim),
                                               ge.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return grad_prim, ge

    def tangent(self, prim0: torch.Tensor, dprim0: Optional[torch.Tensor], eos: np.ndarray,
                deos: Optional[np.ndarray], dts: np.ndarray, want_state: bool = False):
        """The directional derivative of the final state (tj_tangent) along
        dprim0 (same layout as prim0, None: zero) and deos ((M,
        TJ_MAX_EOS_PARAMS), None: zero), from the same FP64 update as
        forward(). Returns (state or None, dstate) on prim0's device."""
        prim0 = prim0.detach().contiguous().to(torch.float64)
        dp = None if dprim0 is None else dprim0.detach().contiguous().to(torch.float64)
        eos = np.ascontiguousarray(eos, dtype=np.float64)
        de = None if deos is None else np.ascontiguousarray(deos, dtype=np.float64)
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        if prim0.is_cuda:
            torch.cuda.current_stream().synchronize()
        st = torch.empty(self.shape_state, dtype=torch.float64, device=prim0.device) if want_state else None
        ds = torch.empty(self.shape_state, dtype=torch.float64, device=prim0.device)
        dptr = lambda a: None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self.sim._check(self.sim.L.tj_tangent(self.sim.h, 0, _ptr(prim0), None if dp is None else _ptr(dp),
                                              dptr(eos), dptr(de), len(dts), dptr(dts),
                                              None if st is None else _ptr(st), _ptr(ds)))
        return st, ds

    def close(self):
        self.sim.close()


class TenjinRun(torch.autograd.Function):
    """state = TenjinRun.apply(prim0, eos, run, dts, stride)

    prim0: (nprim, nz, ny, nx) float64 tensor; eos: (M, TJ_MAX_EOS_PARAMS)
    float64 tensor (CPU). Returns the final state (ncomp, nz, ny, nx) on
    prim0's device. Backward returns the gradients of prim0 and eos."""

    @staticmethod
    def forward(ctx, prim0, eos, run: AdjointRun, dts, stride: int):
        ctx.run = run
        ctx.eos_device = eos.device
        return run.forward(prim0, eos.detach().cpu().numpy(), np.asarray(dts), stride)

    @staticmethod
    def backward(ctx, grad_state):
        gp, ge = ctx.run.backward(grad_state)
        gp = gp if ctx.needs_input_grad[0] else None
        ge = torch.from_numpy(ge).to(ctx.eos_device) if ctx.needs_input_grad[1] else None
        return gp, ge, None, None, None


def eos_vector(gamma: torch.Tensor, p_inf: torch.Tensor, rest: torch.Tensor) -> torch.Tensor:
    """Raw stiffened-gas parameter rows [gamma, -gamma p_inf, e_ref, CV, 0...]
    from per-material gamma, p_inf and the remaining (e_ref, CV) columns."""
    cols = [gamma, -gamma * p_inf, rest[:, 0], rest[:, 1]]
    pad = torch.zeros(gamma.shape[0], MAX_EOS - 4, dtype=gamma.dtype, device=gamma.device)
    return torch.cat([torch.stack(cols, dim=1), pad], dim=1)


def density_misfit(state: torch.Tensor, target: torch.Tensor, M: int, cell_area: float) -> torch.Tensor:
    """J = 1/2 sum over cells (rho - rho_target)^2 dx dy with rho = sum_m alphaRho_m."""
    rho = state[M:2 * M].sum(dim=0)
    return 0.5 * ((rho - target) ** 2).sum() * cell_area


def interface_problem_check(n: int = 512, nsteps: int = 200, stride: int = 20, ndir: int = 64,
                            step_rho: float = 1e-8, step_eos: float = 1e-8, seed: int = 0,
                            background: float = 1e-3, tlm_dirs: int = 0) -> dict:
    """The adjoint on the 2-D water/air interface problem: n^2 cells, nsteps
    steps with the dt schedule of a plain FP64 run, checkpoints every
    `stride` steps, J = 1/2 sum (rho - rho_target)^2 dx^2 with rho_target =
    rho_final (1 + 0.01 N(0,1)) (seeded). Times tj_forward and tj_backward
    (each returns after its stream has drained) and compares the gradient with
    central differences of the same forward on `ndir` seeded directions in
    the space of the initial partial densities (smooth fields) and the EOS
    parameters (gamma, p_ref) of both materials. The base state carries a
    smooth background of relative amplitude `background` (the limiter has no
    derivative at an exactly uniform state). Each direction is checked as the
    sum of its two parts, each differenced with its own relative step:
    `step_rho` along the partial densities and `step_eos` along the EOS
    parameters. Along both, central differences straddle the kinks of the
    discrete choices (limiter, BVD-THINC, wave-speed maxima, HLLC side) of
    cells whose margin is below the step, an error that falls with the step:
    at 128^2 and 60 steps the EOS part goes from 4e-5 at 1e-6 to 3e-6 at 1e-8
    while rounding stays below 1e-6.

    `tlm_dirs` further directions (the same kind) are checked against the
    tangent-linear run (tj_tangent): <grad_state, dstate> against
    <grad_prim0, dprim0> + <grad_eos, deos>. Both differentiate the branches
    the FP64 run takes, so they agree to rounding with or without the
    background, where central differences cannot."""
    import time

    from . import cases

    c = cases.shock_bubble_2d(n=n, max_grid_size=min(128, n), thinc=1, background=background)
    M = c.M
    area = (1.0 / n) ** 2
    run = AdjointRun(c)
    dts = run.dt_schedule(nsteps)
    prim = torch.from_numpy(np.ascontiguousarray(c.domains[0].prim)).cuda()
    eos = run.eos_array()
    rng = np.random.default_rng(seed)
    out = run.forward(prim, eos, dts, stride)
    rho = out[M:2 * M].sum(dim=0)
    target = rho * torch.from_numpy(1 + 0.01 * rng.standard_normal(tuple(rho.shape))).cuda()
    gs = torch.zeros_like(out)
    gs[M:2 * M] = ((rho - target) * area).unsqueeze(0)
    gp_dev = torch.empty(run.shape_prim, dtype=torch.float64, device="cuda")
    run.backward(gs, gp_dev)  # warm-up of both directions
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run.forward(prim, eos, dts, stride, out=out)
    t1 = time.perf_counter()
    gp, ge = run.backward(gs, gp_dev)
    t2 = time.perf_counter()
    fwd_s, bwd_s = t1 - t0, t2 - t1
    gp = gp.cpu().numpy()
    prim0 = prim.cpu().numpy()

    def J(p, e):
        o = run.forward(torch.from_numpy(p).cuda(), e, dts, nsteps)
        return float(density_misfit(o, target, M, area))

    def central(v, ve, h):
        return (J(prim0 + h * v, eos + h * ve) - J(prim0 - h * v, eos - h * ve)) / (2 * h)

    def direction(r):
        v = np.zeros_like(prim0)
        for m in range(M):
            v[M + m, 0] = cases.smooth_field(r, n) * prim0[M + m, 0]
        ve = np.zeros_like(eos)
        ve[:, 0:2] = r.standard_normal((M, 2)) * eos[:, 0:2]
        return v, ve

    tlm = None
    if tlm_dirs > 0:
        gsn = gs.cpu().numpy()
        terrs = []
        ts = []
        rng_t = np.random.default_rng(seed + 1000)
        for _ in range(tlm_dirs):
            v, ve = direction(rng_t)
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            _, ds = run.tangent(prim, torch.from_numpy(v).cuda(), eos, ve, dts)
            ts.append(time.perf_counter() - t3)
            tl = float((gsn * ds.cpu().numpy()).sum())
            ad = float((gp * v).sum() + (ge * ve).sum())
            terrs.append(abs(tl - ad) / max(abs(tl), abs(ad)))
        e = np.array(terrs)
        tlm = {"directions": tlm_dirs, "max_rel_err": float(e.max()), "median_rel_err": float(np.median(e)),
               "frac_within_1e-9": float((e <= 1e-9).mean()), "tangent_run_s": float(np.median(ts))}

    errs, errs_rho, errs_eos = [], [], []
    for _ in range(ndir):
        v, ve = direction(rng)
        fd_r, ad_r = central(v, np.zeros_like(eos), step_rho), float((gp * v).sum())
        fd_e, ad_e = central(np.zeros_like(prim0), ve, step_eos), float((ge * ve).sum())
        errs_rho.append(abs(fd_r - ad_r) / max(abs(fd_r), abs(ad_r)))
        errs_eos.append(abs(fd_e - ad_e) / max(abs(fd_e), abs(ad_e)))
        fd, ad = fd_r + fd_e, ad_r + ad_e
        errs.append(abs(fd - ad) / max(abs(fd), abs(ad)))
    run.close()

    def summary(e):
        e = np.array(e)
        if not e.size:
            return None
        return {"max_rel_err": float(e.max()), "median_rel_err": float(np.median(e)),
                "frac_within_1e-5": float((e <= 1e-5).mean())}

    fd = {"directions": ndir, "step_rho": step_rho, "step_eos": step_eos, "combined": summary(errs),
          "rho_part": summary(errs_rho), "eos_part": summary(errs_eos)} if ndir > 0 else None
    return {"workload": f"2-D water/air interface, {n}x{n}, {nsteps} steps, THINC, checkpoint every {stride}",
            "forward_s": fwd_s, "backward_s": bwd_s, "ratio": bwd_s / fwd_s,
            "forward_cell_updates_per_s": n * n * nsteps / fwd_s, "fd_check": fd, "tangent_check": tlm,
            "inputs": "initial rho_k fields (smooth seeded directions) and gamma, p_ref of both materials",
            "base_background": background}


def general_check(name: str = "copper", n: int = 24, nsteps: int = 4, stride: int = 2, ndir: int = 8,
                  seed: int = 0) -> dict:
    """The general reverse mode (tj_forward / tj_backward on a configuration
    the 2-D fluid adjoint does not cover) against the tangent-linear run:
    forward and backward times, and |<w, tangent(v, ve)> - (<grad_prim0, v>
    + <grad_eos, ve>)| relative, over `ndir` seeded white-noise directions
    of the primitives and the EOS parameters and a seeded gradient w on the
    final carried words. `name`: "copper" (3-D copper plate, n^3, 5-wave
    solver, plastic radial return, cleanUpV) or "sod" (1-D shock tube, n
    cells)."""
    import time

    from . import cases
    from .host import carried_components

    if name == "copper":
        c = cases.copper_plate_3d(n=n, max_grid_size=n)
        workload = f"copper plate {n}^3, {nsteps} steps, checkpoint every {stride}"
    else:
        c = cases.sod_1d(ncells=n, max_grid_size=n)
        workload = f"1-D shock tube, {n} cells, {nsteps} steps, checkpoint every {stride}"
    run = AdjointRun(c)
    dts = run.dt_schedule(nsteps)
    prim0 = np.ascontiguousarray(c.domains[0].prim)
    prim = torch.from_numpy(prim0).cuda()
    eos = run.eos_array()
    rng = np.random.default_rng(seed)
    out = run.forward(prim, eos, dts, stride)
    carried = carried_components(c)
    w = np.zeros(run.shape_state)
    w[carried] = rng.standard_normal((len(carried),) + run.shape_state[1:])
    scale = np.abs(out.cpu().numpy()).reshape(out.shape[0], -1).max(axis=1)
    w /= np.where(scale > 0, scale, 1.0)[:, None, None, None]
    wt = torch.from_numpy(w).cuda()
    run.backward(wt)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run.forward(prim, eos, dts, stride)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    gp, ge = run.backward(wt)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    gp = gp.cpu().numpy()
    errs = []
    for _ in range(ndir):
        v = rng.standard_normal(prim0.shape) * np.abs(prim0) * 1e-3
        ve = np.zeros_like(eos)
        for m, mat in enumerate(c.materials):
            ve[m, :len(mat.params)] = rng.standard_normal(len(mat.params)) * np.abs(eos[m, :len(mat.params)]) * 1e-3
        _, ds = run.tangent(prim, torch.from_numpy(v).cuda(), eos, ve, dts)
        tl = float((w * ds.cpu().numpy()).sum())
        ad = float((gp * v).sum() + (ge * ve).sum())
        errs.append(abs(tl - ad) / max(abs(tl), abs(ad)))
    run.close()
    e = np.array(errs)
    return {"workload": workload, "forward_s": t1 - t0, "backward_s": t2 - t1, "ratio": (t2 - t1) / (t1 - t0),
            "tangent_check": {"directions": ndir, "max_rel_err": float(e.max()),
                              "median_rel_err": float(np.median(e))}}


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser(description="adjoint timing and finite-difference check")
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--stride", type=int, default=20)
    ap.add_argument("--dirs", type=int, default=64)
    ap.add_argument("--step-rho", type=float, default=1e-8, help="relative step along the partial densities")
    ap.add_argument("--step-eos", type=float, default=1e-8, help="relative step along (gamma, p_ref)")
    ap.add_argument("--tlm-dirs", type=int, default=0, help="directions checked against the tangent-linear run")
    ap.add_argument("--background", type=float, default=1e-3,
                    help="relative amplitude of the smooth background of the base state (0: the configuration as "
                         "stated, with exactly uniform regions)")
    ap.add_argument("--general", choices=["copper", "sod"], default=None,
                    help="check the general reverse mode on this case instead (--n cells per axis)")
    a = ap.parse_args()
    from . import build
    build.build()
    if a.general:
        print(json.dumps(general_check(a.general, a.n, a.steps, a.stride, a.dirs)))
    else:
        print(json.dumps(interface_problem_check(a.n, a.steps, a.stride, a.dirs, step_rho=a.step_rho,
                                                 step_eos=a.step_eos, background=a.background, tlm_dirs=a.tlm_dirs)))
