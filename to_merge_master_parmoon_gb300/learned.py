"""Learned per-cell smoother: network handle, training-pair harvest and the
training loop (AdamW, mini-batches) around the library's GPU kernels.

The network (397 -> 256 -> 256 -> 85, GELU, BF16 tensor-core GEMMs with FP32
accumulation) and every forward/backward/update step run in libpmgpu; this
module only orders the calls.  Device buffers for the training set are torch
tensors (plumbing).
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from ._lib import gpu_lib
from .solver import PmError, PmSolver

N_IN, N_HIDDEN, N_OUT = 397, 256, 85
FEATURE_CLAMP = 1.0e3  # |feature| bound of the feature kernel (kFeatureClamp)


def _torch_done(t):
    """Wait for the work torch has queued on its current stream of t's device:
    the library runs on its own stream, so tensors that torch has just
    written (index_select, randperm, empty from recycled memory) must be
    complete before a library kernel reads or writes them."""
    import torch
    torch.cuda.current_stream(t.device).synchronize()


class Mlp:
    def __init__(self, device: int = 0, seed: int = 0, max_batch: int = 8192):
        self._lib = gpu_lib()
        h = C.c_void_p()
        st = self._lib.pm_mlp_create(C.byref(h), device, seed, max_batch)
        if st != 0:
            raise PmError(st, "pm_mlp_create")
        self._h = h
        self.max_batch = max_batch
        self.n_params = self._lib.pm_mlp_num_params()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pm_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def params(self) -> np.ndarray:
        p = np.empty(self.n_params, np.float32)
        st = self._lib.pm_mlp_get_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float)), p.size)
        if st != 0:
            raise PmError(st, "pm_mlp_get_params")
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        st = self._lib.pm_mlp_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float)), p.size)
        if st != 0:
            raise PmError(st, "pm_mlp_set_params")

    def set_tensor_path(self, tcgen05: bool):
        """The GEMMs (forward and training) on tcgen05 (True, the default) or
        mma.sync (False)."""
        st = self._lib.pm_mlp_set_tensor_path(self._h, int(tcgen05))
        if st != 0:
            raise PmError(st, "pm_mlp_set_tensor_path")

    def forward(self, X):
        """X: torch float32 cuda tensor [M, 397] -> [M, 85]."""
        import torch
        Y = torch.empty((X.shape[0], N_OUT), dtype=torch.float32, device=X.device)
        _torch_done(X)
        st = self._lib.pm_mlp_forward(self._h, C.c_void_p(X.data_ptr()), X.shape[0],
                                      C.c_void_p(Y.data_ptr()))
        if st != 0:
            raise PmError(st, "pm_mlp_forward")
        return Y

    def loss_grad(self, X, T, want_grad: bool = False):
        loss = C.c_double()
        g = np.empty(self.n_params, np.float32) if want_grad else None
        _torch_done(X)
        st = self._lib.pm_mlp_loss_grad(self._h, C.c_void_p(X.data_ptr()), C.c_void_p(T.data_ptr()),
                                        X.shape[0], C.byref(loss),
                                        g.ctypes.data_as(C.POINTER(C.c_float)) if g is not None else None)
        if st != 0:
            raise PmError(st, "pm_mlp_loss_grad")
        return (loss.value, g) if want_grad else loss.value

    def adamw(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=1e-2):
        st = self._lib.pm_mlp_adamw_step(self._h, lr, beta1, beta2, eps, weight_decay)
        if st != 0:
            raise PmError(st, "pm_mlp_adamw_step")


def harvest_pairs(problems, n_cycles: int = 8, device: int = 0, precision: str = "fp64",
                  max_target_rms: float = 1e4, log=None):
    """(features, scaled error) pairs from the plain solver on each problem's
    finest level: exact solution by FGMRES to 1e-11, then n_cycles V-cycle
    iterations from zero.  Rows that are not finite or whose scaled error has
    an rms above max_target_rms (the plain iteration diverging on strongly
    convective problems) are dropped.  Returns torch tensors X [n, 397],
    T [n, 85]."""
    import torch
    total = sum(P.desc(P.n_levels - 1).n_cells * n_cycles for P in problems)
    X = torch.empty((total, N_IN), dtype=torch.float32, device=f"cuda:{device}")
    T = torch.empty((total, N_OUT), dtype=torch.float32, device=f"cuda:{device}")
    n = 0
    for P in problems:
        b = P.rhs()
        nu3 = 3 * P.desc(P.n_levels - 1).n_udof
        bp = b.copy()
        bp[nu3::4] -= bp[nu3::4].mean()
        r0 = float(np.linalg.norm(bp))
        S = PmSolver(P.descs, precision=precision, device=device, restart=30, maxit=300,
                     res_norm_min=1e-11 * r0)
        xs, info = S.iterate(np.zeros_like(b), b, allow=(0, 1))
        n0 = n
        converged = info["true_res"] <= 1e-9 * r0
        if converged:  # the targets are errors against this solution
            _torch_done(X)
            n = S.harvest(xs, b, n_cycles, X.data_ptr(), T.data_ptr(), total, n)
        S.close()
        if log:
            log(f"harvest nu={P.nu:.2e}: exact solve {info['iterations']} it "
                f"(rel {info['true_res'] / r0:.1e}), {n - n0} rows"
                + ("" if converged else " (skipped: not converged)"))
    X, T = X[:n], T[:n]
    keep = torch.isfinite(X).all(1) & torch.isfinite(T).all(1)
    keep &= T.pow(2).mean(1).sqrt() <= max_target_rms
    # cells at the feature clamp (own residual ~0 against their neighbours')
    keep &= X.abs().amax(1) < 0.999 * FEATURE_CLAMP
    return X[keep].contiguous(), T[keep].contiguous()


def harvest_manufactured(problems, n_cycles: int = 8, device: int = 0, noise: float = 0.1,
                         seed: int = 0, max_target_rms: float = 1e4, solutions=None, log=None):
    """(features, scaled error) pairs with a manufactured solution on each
    problem's finest level: u* = a smooth divergence-free field (the nodal
    convection field of a problem with another seed) plus `noise` times
    seeded white noise on every DOF (or solutions[k] when given), right-hand
    side b := K u* (the library's FP64 mat-vec), so the error u* - u of the
    plain iterates is known without an exact solve, also where the plain
    solver does not converge (strongly convective nu).  Same filters and
    output as harvest_pairs."""
    import torch
    from .problem import OseenProblem
    total = sum(P.desc(P.n_levels - 1).n_cells * n_cycles for P in problems)
    X = torch.empty((total, N_IN), dtype=torch.float32, device=f"cuda:{device}")
    T = torch.empty((total, N_OUT), dtype=torch.float32, device=f"cuda:{device}")
    n = 0
    rng = np.random.default_rng(seed)
    for k, P in enumerate(problems):
        L = P.n_levels
        S = PmSolver(P.descs, precision="fp64", device=device)
        nu3 = 3 * P.desc(L - 1).n_udof
        if solutions is not None:
            us = np.ascontiguousarray(solutions[k], dtype=np.float64)
        else:
            Q = OseenProblem(n_levels=L, nu=P.nu, seed=5000 + k)
            us = np.zeros(P.ndof(-1))
            us[:nu3] = Q.convection_nodal(L - 1)
            us += noise * rng.standard_normal(us.size)
        b = S.matvec(L - 1, us)
        n0 = n
        _torch_done(X)
        n = S.harvest(us, b, n_cycles, X.data_ptr(), T.data_ptr(), total, n)
        S.close()
        if log:
            log(f"manufactured harvest nu={P.nu:.2e}: {n - n0} rows")
    X, T = X[:n], T[:n]
    keep = torch.isfinite(X).all(1) & torch.isfinite(T).all(1)
    keep &= T.pow(2).mean(1).sqrt() <= max_target_rms
    keep &= X.abs().amax(1) < 0.999 * FEATURE_CLAMP
    return X[keep].contiguous(), T[keep].contiguous()


def train(mlp: Mlp, X, T, epochs: int = 20, batch: int = 4096, lr: float = 1e-3,
          weight_decay: float = 1e-2, seed: int = 0, log=None):
    """AdamW mini-batch training on device tensors; returns per-epoch mean loss."""
    import torch
    g = torch.Generator(device=X.device)
    g.manual_seed(seed)
    n = X.shape[0]
    batch = min(batch, mlp.max_batch)
    hist = []
    t0 = time.time()
    for ep in range(epochs):
        perm = torch.randperm(n, device=X.device, generator=g)
        tot, cnt = 0.0, 0
        for s in range(0, n - batch + 1, batch):
            idx = perm[s:s + batch]
            xb = X.index_select(0, idx).contiguous()
            tb = T.index_select(0, idx).contiguous()
            loss = mlp.loss_grad(xb, tb)
            mlp.adamw(lr=lr, weight_decay=weight_decay)
            tot += loss
            cnt += 1
        hist.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4e} ({time.time() - t0:.1f}s)")
    return hist


def relative_loss(mlp: Mlp, X, T, batch: int = 8192) -> float:
    """||pred - T||^2 / ||T||^2 over a data set (1.0 = predicting zero)."""
    num = den = 0.0
    batch = min(batch, mlp.max_batch)
    for s in range(0, X.shape[0], batch):
        xb = X[s:s + batch].contiguous()
        y = mlp.forward(xb)
        tb = T[s:s + batch]
        num += float(((y - tb) ** 2).sum())
        den += float((tb ** 2).sum())
    return num / max(den, 1e-300)


# the benchmark's training configuration: pairs harvested from plain FP64
# solves of 32^3 problems (5 levels) with nu log-uniform in [1e-3, 1e-1]
# (seeds 1000+k), 8 cycles each, AdamW lr 1e-3, 20 epochs of batches of 4096
STANDARD_CONFIG = dict(levels=5, problems=8, cycles=8, epochs=20, batch=4096, lr=1e-3, seed=0,
                       nu_range=(1e-3, 1e-1), features="neighbourhood-max-rms")


def standard_network(device: int = 0, problems: int | None = None, cache_dir=None, log=None):
    """The network of STANDARD_CONFIG (``problems`` overrides the number of
    harvested problems), trained on the GPU; with ``cache_dir`` the weights
    are kept there keyed by the configuration.  Returns (Mlp, info dict)."""
    import hashlib
    import json
    from pathlib import Path

    from .problem import OseenProblem
    cfg = dict(STANDARD_CONFIG)
    if problems is not None:
        cfg["problems"] = problems
    key = hashlib.sha1(json.dumps(cfg, sort_keys=True).encode()).hexdigest()[:12]
    cache = Path(cache_dir) / f"mlp_{key}.npy" if cache_dir is not None else None
    net = Mlp(device=device, seed=cfg["seed"], max_batch=cfg["batch"])
    info = {"config": cfg, "cached": bool(cache is not None and cache.exists())}
    if info["cached"]:
        net.set_params(np.load(cache))
        return net, info
    rng = np.random.default_rng(cfg["seed"])
    lo, hi = np.log10(cfg["nu_range"][0]), np.log10(cfg["nu_range"][1])
    t = time.perf_counter()
    probs = [OseenProblem(n_levels=cfg["levels"], nu=float(10 ** rng.uniform(lo, hi)),
                          seed=1000 + k) for k in range(cfg["problems"])]
    X, T = harvest_pairs(probs, n_cycles=cfg["cycles"], device=device, log=log)
    info["harvest_s"] = time.perf_counter() - t
    info["pairs"] = int(X.shape[0])
    t = time.perf_counter()
    hist = train(net, X, T, epochs=cfg["epochs"], batch=cfg["batch"], lr=cfg["lr"],
                 seed=cfg["seed"])
    info["train_s"] = time.perf_counter() - t
    info["loss_first_last"] = [hist[0], hist[-1]]
    info["relative_loss"] = relative_loss(net, X, T)
    if cache is not None:
        cache.parent.mkdir(parents=True, exist_ok=True)
        np.save(cache, net.params())
    del X, T
    return net, info
