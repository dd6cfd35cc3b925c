"""Flexible CG with the learned U-Net preconditioner, its training data and
training loop (the learned-preconditioner case of the Poisson benchmark).

* Training data are residual/error pairs the solver itself produces: for
  seeded Gaussian random right-hand sides with a k^-2 power spectrum (zero on
  the Dirichlet faces), plain CG runs to convergence and the pairs
  (r_k, x_final - x_k) are kept at a fixed set of iterations k.
* Training minimises |M(r) - e|^2 / |e|^2 with Adam on the U-Net's FP32
  master weights (forward/backward on the tensor-core kernels).
* The solver is FCG(1) (flexible CG with one-step A-orthogonalisation, which
  tolerates a nonlinear preconditioner): z = M(r) masked to the Free rows
  and followed by damped-Jacobi sweeps on A z = r,
  p = z - (z.q_prev / p_prev.q_prev) p_prev, q = A p, alpha = p.r / p.q;
  x accumulates in FP64 and the true residual b - A x is recomputed in FP64
  every `refresh` iterations. If the true residual fails to halve over
  `stall` iterations the solve continues with Jacobi-PCG (ngb_cg_solve) from
  the current x.
"""
import math
import time

import torch

from . import (STORE_F32, STORE_F64, _ptr, cg_solve, cg_workspace, check, dot, laplacian_apply, lib, mg_apply, mg_jacobi,
                mg_prolong_add, mg_residual, mg_restrict, poisson_desc)


def free_mask(n, device):
    m = torch.zeros(n, n, n, dtype=torch.float32, device=device)
    m[1:-1, 1:-1, 1:-1] = 1.0
    return m.reshape(-1)


def grf_k2(n, seed, device):
    """Gaussian random field with power spectrum |k|^-2 (amplitude |k|^-1), zero on the box faces, unit RMS."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    white = torch.randn(n, n, n, generator=g).to(device)
    F = torch.fft.rfftn(white)
    kz = torch.fft.fftfreq(n, device=device).reshape(n, 1, 1)
    ky = torch.fft.fftfreq(n, device=device).reshape(1, n, 1)
    kx = torch.fft.rfftfreq(n, device=device).reshape(1, 1, n // 2 + 1)
    k = torch.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    k[0, 0, 0] = 1.0
    field = torch.fft.irfftn(F / k, s=(n, n, n)).reshape(-1)
    field = field * free_mask(n, device)
    return (field / field.pow(2).mean().sqrt()).float()


class _Ops:
    """A, dot on the device through the C ABI (FP32 and FP64 fields)."""

    def __init__(self, n, device):
        self.n = n
        self.dev = device
        self.d32 = poisson_desc(n, n, n, "f32", 1.0)
        self.d64 = poisson_desc(n, n, n, "f64", 1.0)
        self.res = torch.zeros(1, dtype=torch.float64, device=device)
        self.scratch = torch.empty(lib().ngb_dot_scratch_doubles(n ** 3), dtype=torch.float64, device=device)

    def A(self, u, out):
        laplacian_apply(self.d64 if u.dtype == torch.float64 else self.d32, u, out)
        return out

    def dot(self, a, b):
        dot(a, b, self.res, self.scratch)
        return float(self.res.item())


def cg_pairs(n, seed, captures, device, tol=1e-7, max_iter=5000):
    """Plain CG on A x = b (b = k^-2 field); returns [(r_k, x_final - x_k)] at iterations `captures`."""
    ops = _Ops(n, device)
    b = grf_k2(n, seed, device)
    x = torch.zeros_like(b)
    r = b.clone()
    p = r.clone()
    q = torch.empty_like(b)
    rr = ops.dot(r, r)
    bb = rr
    saved = {}
    for k in range(max_iter):
        if k in captures:
            saved[k] = (r.clone(), x.clone())
        ops.A(p, q)
        alpha = rr / ops.dot(p, q)
        x.add_(p, alpha=alpha)
        r.add_(q, alpha=-alpha)
        rr_new = ops.dot(r, r)
        if rr_new <= tol * tol * bb:
            break
        p.mul_(rr_new / rr).add_(r)
        rr = rr_new
    return [(rk, x - xk) for rk, xk in saved.values()]


def make_training_set(n=128, systems=200, captures=(2, 5, 10, 20, 40, 80, 120, 160, 200, 250), seed=2024,
                      device="cuda", count=None):
    """Solver pairs from `systems` seeded systems, or, with `count`, from as
    many systems as it takes to reach exactly `count` pairs (a CG run that
    converges before a capture point yields fewer pairs)."""
    pairs = []
    s = 0
    while (s < systems) if count is None else (len(pairs) < count):
        pairs += cg_pairs(n, seed + s, set(captures), device)
        s += 1
    return pairs if count is None else pairs[:count]


def train(net, pairs, epochs=2, lr=1e-3, log=None, seed=0):
    """Adam on the relative loss |M(r) - e|^2 / |e|^2 of each pair, one pair
    per step. The step stays on the device (input scale, loss and gradient
    scale as device scalars, no tensor-core time-out check inside the epoch):
    the host reads the losses and checks the convolutions once per epoch."""
    g = torch.Generator().manual_seed(seed)
    losses = []
    for ep in range(epochs):
        order = torch.randperm(len(pairs), generator=g).tolist()
        step_losses = []
        for i in order:
            r, e = pairs[i]
            z = net.forward(r, sync=False)
            ee = (e.double() ** 2).sum()
            diff = z - e
            step_losses.append((diff.double() ** 2).sum() / ee)
            net.zero_grad()
            net.backward((2.0 / ee).float() * diff, sync=False)
            net.adam_step(lr=lr)
        net.check()
        losses += torch.stack(step_losses).tolist()
        if log:
            log("epoch %d: mean relative loss %.4f" % (ep, sum(losses[-len(pairs):]) / len(pairs)))
    return losses


def fcg_solve(net, b, x, tol=1e-8, max_iter=2000, refresh=10, stall=20, fallback=True, ws=None, smooth=2,
              omega=2.0 / 3.0):
    """FCG(1) with z = M(r) from the network on the fine grid. b: float32 n^3
    field (zero on the faces); x: float64 n^3 initial guess / result.

    The network's output carries white rounding noise from its BF16
    activations at about 1e-3 of |z|; A amplifies it by up to 12 while
    |z| / |r| reaches 1 / lambda_min, so the injected residual is as large as
    the residual itself and FCG stalls. `smooth` damped-Jacobi sweeps
    z += omega D^-1 (r - A z) after the network remove that high-frequency
    error (each sweep scales it by at most 1/3 for omega = 2/3)."""
    n = round(b.numel() ** (1.0 / 3.0))
    ops = _Ops(n, b.device)
    mask = free_mask(n, b.device)
    az = torch.empty_like(b)

    def precondition(r):
        z = net.forward(r) * mask
        ops.A(z, az)
        for _ in range(smooth):
            z.add_((r - az) * mask, alpha=omega / 6.0)
            ops.A(z, az)
        return z, az.clone()

    return _fcg(precondition, ops, mask, b, x, tol, max_iter, refresh, stall, fallback, ws)


class VCycle:
    """Multilevel preconditioner z = M(r) whose coarsest-level solve is the network.

    Levels l = 0..L are vertex-centred grids of n / 2^l nodes with spacing
    2^l (ngb_mg_* kernels). On every level above the coarsest: two damped
    Jacobi sweeps from zero, the residual, full-weighting restriction; on the
    coarsest level the correction e_L solves A_{2^L} e_L = r_L, which is
    A_1 e_L = 4^L r_L, the problem the network was trained on (A with unit
    spacing): e_L = 4^L M(r_L); then trilinear prolongation and `post` Jacobi
    sweeps back up. The smoothing levels remove the high-frequency error the
    BF16 network output carries and the network supplies the smooth
    components Jacobi cannot reach; the network's correction enters with the
    energy-minimising step on the coarsest level. `coarse="none"` drops the
    coarsest correction (the same cycle without the network)."""

    def __init__(self, n, levels, net=None, coarse="net", omega=6.0 / 7.0, post=2, device="cuda"):
        if coarse not in ("net", "none"):
            raise ValueError("coarse must be 'net' or 'none'")
        if coarse == "net" and net is None:
            raise ValueError("coarse='net' needs a network")
        if n % (1 << levels) != 0 or (n >> levels) < 8:
            raise ValueError("n must be divisible by 2^levels with at least 8 nodes on the coarsest level")
        self.n, self.levels, self.net, self.coarse = n, levels, net, coarse
        self.omega, self.post = omega, post
        self.descs = [poisson_desc(n >> l, n >> l, n >> l, "f32", float(1 << l)) for l in range(levels + 1)]
        f32 = dict(dtype=torch.float32, device=device)
        self.u = [torch.empty((n >> l) ** 3, **f32) for l in range(levels)]
        self.tmp = [torch.empty((n >> l) ** 3, **f32) for l in range(levels)]
        self.res = [torch.empty((n >> l) ** 3, **f32) for l in range(levels)]
        self.r = [None] + [torch.empty((n >> l) ** 3, **f32) for l in range(1, levels + 1)]
        self.coarse_mask = free_mask(n >> levels, device)
        nc3 = (n >> levels) ** 3
        self.e_coarse, self.ae_coarse = torch.empty(nc3, **f32), torch.empty(nc3, **f32)
        self.scal = torch.zeros(3, dtype=torch.float64, device=device)  # |r|^2, <e, r>, <e, A e>
        self.scratch = torch.empty(lib().ngb_dot_scratch_doubles(nc3), dtype=torch.float64, device=device)

    def __call__(self, r):
        z = torch.empty_like(r)
        return self._cycle(0, r, z)

    def _cycle(self, l, r, out=None):
        if l == self.levels:
            return None if self.coarse == "none" else self._coarse_solve(l, r)
        d = self.descs[l]
        u = self.u[l] if out is None else out
        mg_jacobi(d, None, r, u, self.omega)
        mg_residual(d, u, r, self.res[l])
        mg_restrict(d, self.res[l], self.r[l + 1], 1.0)
        e = self._cycle(l + 1, self.r[l + 1])
        if e is not None:
            mg_prolong_add(d, e, u)
        a, b = u, self.tmp[l]
        for _ in range(self.post):
            mg_jacobi(d, a, r, b, self.omega)
            a, b = b, a
        if a is not u:
            u.copy_(a)
        return u

    def _coarse_solve(self, l, r):
        """e = beta 4^l M(r): the network's answer to A_1 e = 4^l r, scaled by
        the step beta = <e, r> / <e, A e> that minimises the coarse-level
        error energy along e (0 when e is not a descent direction, so a poor
        network output cannot make the cycle worse than the cycle without it).
        Device-side library calls only: no host synchronisation."""
        e, ae, s = self.e_coarse, self.ae_coarse, self.scal
        self.net.apply(r, e, float(4 ** l), s[0:1], self.scratch)
        mg_apply(self.descs[l], e, ae)
        dot(e, r, s[1:2], self.scratch)
        dot(e, ae, s[2:3], self.scratch)
        check(lib().ngb_scale_by_ratio(e.numel(), _ptr(e), _ptr(s[1:2]), _ptr(s[2:3]), None))
        return e


def fcg_solve_vcycle(vcycle, b, x, tol=1e-8, max_iter=2000, refresh=10, stall=30, fallback=True, ws=None):
    """FCG(1) preconditioned by a VCycle (network on the coarsest level)."""
    n = round(b.numel() ** (1.0 / 3.0))
    ops = _Ops(n, b.device)
    mask = free_mask(n, b.device)

    def precondition(r):
        z = vcycle(r)
        az = torch.empty_like(z)
        mg_apply(vcycle.descs[0], z, az)
        return z, az

    net = vcycle.net if vcycle.coarse == "net" else None
    return _fcg(precondition, ops, mask, b, x, tol, max_iter, refresh, stall, fallback, ws,
                check_net=net.check if net is not None else None)


def _fcg(precondition, ops, mask, b, x, tol, max_iter, refresh, stall, fallback, ws, check_net=None):
    """FCG(1): p = z - (z.q_prev / p_prev.q_prev) p_prev, q = A p, alpha = p.r / p.q;
    x in FP64, the true residual b - A x recomputed in FP64 every `refresh`
    iterations; Jacobi-PCG takes over when it fails to halve over `stall`.
    The vector steps and their sums run in ngb_fcg_direction / ngb_fcg_update
    with device scalars: one host read (|r|) per iteration."""
    n = ops.n
    dev = b.device
    L = lib()
    t0 = time.perf_counter()
    bn = ops.dot(b, b) ** 0.5
    ax = torch.empty_like(x)
    mask64 = mask.double()
    N = b.numel()
    scratch = torch.empty(L.ngb_fcg_scratch_doubles(N), dtype=torch.float64, device=dev)
    scal = torch.zeros(8, dtype=torch.float64, device=dev)  # zq, rr, (pq, pr) x 2 alternating

    def true_residual():
        ops.A(x, ax)
        rt = (b - ax).mul_(mask64)
        return rt.float(), ops.dot(rt, rt) ** 0.5 / bn

    r, rel = true_residual()
    history = [rel]
    p_prev = q_prev = None
    it = 0
    used_fallback = False
    while rel > tol and it < max_iter:
        z, az = precondition(r)
        cur, prev = scal[2 + 2 * (it % 2):4 + 2 * (it % 2)], scal[2 + 2 * ((it + 1) % 2):4 + 2 * ((it + 1) % 2)]
        if p_prev is not None:
            dot(z, q_prev, scal[0:1], ops.scratch)
            check(L.ngb_fcg_direction(N, _ptr(z), _ptr(az), _ptr(p_prev), _ptr(q_prev), _ptr(r), _ptr(scal[0:1]), _ptr(prev),
                                      _ptr(cur), _ptr(scratch), None))
        else:
            check(L.ngb_fcg_direction(N, _ptr(z), _ptr(az), None, None, _ptr(r), None, None, _ptr(cur), _ptr(scratch), None))
        check(L.ngb_fcg_update(N, _ptr(x), _ptr(z), _ptr(r), _ptr(az), _ptr(cur), _ptr(scal[1:2]), _ptr(scratch), None))
        p_prev, q_prev = z, az
        it += 1
        if it % refresh == 0:
            if check_net is not None:
                check_net()
            r, rel = true_residual()
            history.append(rel)
            if fallback and len(history) > stall // refresh and history[-1] > 0.5 * history[-1 - stall // refresh]:
                used_fallback = True
                break
        else:
            rel = float(scal[1].item()) ** 0.5 / bn
        if not math.isfinite(rel):
            # breakdown (p.q zero or not finite): Jacobi-PCG takes over from
            # x if it is still finite, else from zero
            used_fallback = True
            if not bool(torch.isfinite(x).all()):
                x.zero_()
            rel = float("inf")
            break
    if check_net is not None:
        check_net()
    torch.cuda.synchronize()
    extra = {"iterations": 0}
    if used_fallback and rel > tol:
        d = poisson_desc(n, n, n, "f32", 1.0)
        ws = ws if ws is not None else cg_workspace(d, dev)
        extra = cg_solve(d, b, x, ws, tol=tol, max_iter=20000, refresh_every=50, check_every=50, jacobi=True)
        r, rel = true_residual()
    torch.cuda.synchronize()
    return {"iterations": it, "fallback_iterations": extra["iterations"], "fallback": used_fallback,
            "rel_residual": rel, "converged": rel <= tol, "seconds": time.perf_counter() - t0, "history": history}
