"""Run one operation of the library on seeded synthetic inputs and time it.

    python -m adrt_gb300.workloads --op bdrt --n 1024 --batch 8 --reps 5

Prints one JSON line: milliseconds per call (CUDA events on the launching
stream, after warm-up), images per second and the algorithmic bandwidth
(compulsory bytes per call / time).  Useful to time a single kernel family
and as the command line under a profiler.

Ops: adrt, bdrt, iadrt, adjoint, adrt_step, bdrt_step, fmg_restriction,
fmg_prolongation, fmg_highpass, iadrt_fmg, ragged, cg, pcg, precond,
interp, unstitch, coords, net_forward, net_train.
"""

from __future__ import annotations

import argparse
import json
import sys

import torch

OPS = ("adrt", "bdrt", "iadrt", "adjoint", "adrt_step", "bdrt_step", "fmg_restriction", "fmg_prolongation",
       "fmg_highpass", "iadrt_fmg", "ragged", "cg", "pcg", "precond", "interp", "unstitch", "coords",
       "net_forward", "net_train")


def _setup(op: str, n: int, batch: int, dtype, dev):
    """Returns (fn, algorithmic bytes per call, images per call)."""
    import adrt_gb300 as adrt
    from adrt_gb300 import core
    from adrt_gb300.data import ellipse_phantoms, uniform_images

    es = 4 if dtype == torch.float32 else 8
    img = uniform_images(batch, n, seed=0, device=dev, dtype=dtype)
    A = 4 * n * (2 * n - 1)
    if op == "adrt":
        return (lambda: adrt.adrt(img)), es * batch * (n * n + A), batch
    y = adrt.adrt(img)
    if op == "bdrt":
        return (lambda: adrt.bdrt(y)), es * batch * 2 * A, batch
    if op == "iadrt":
        return (lambda: adrt.iadrt(y)), es * batch * 2 * A, batch
    if op == "adjoint":
        from adrt_gb300.autograd import _adjoint_raw

        return (lambda: _adjoint_raw(y)), es * batch * (A + n * n), batch
    if op == "adrt_step":
        z = core.adrt_init(img)
        return (lambda: core.adrt_step(z, 0)), es * batch * 2 * A, batch
    if op == "bdrt_step":
        return (lambda: core.bdrt_step(y, 0)), es * batch * 2 * A, batch
    if op == "fmg_restriction":
        from adrt_gb300 import _ops

        return (lambda: _ops.press_fmg_restriction(y)), es * batch * (A + A // 4), batch
    if op == "fmg_prolongation":
        from adrt_gb300 import _ops

        return (lambda: _ops.press_fmg_prolongation(img)), es * batch * 5 * n * n, batch
    if op == "fmg_highpass":
        from adrt_gb300 import _ops

        return (lambda: _ops.press_fmg_highpass(img)), es * batch * 2 * n * n, batch
    if op == "iadrt_fmg":
        return (lambda: core.iadrt_fmg_step(y)), 0, batch
    if op == "ragged":
        from adrt_gb300.data import ragged_phantoms
        from adrt_gb300.ragged import adrt_ragged

        imgs = ragged_phantoms(batch, seed=0, device=dev, dtype=dtype)
        nbytes = sum(es * (m.shape[-1] ** 2 + 4 * m.shape[-1] * (2 * m.shape[-1] - 1)) for m in imgs)
        return (lambda: adrt_ragged(imgs)), nbytes, batch
    if op in ("cg", "pcg"):
        from adrt_gb300 import cg as cgmod
        from adrt_gb300 import precond

        xt = ellipse_phantoms(batch, n, seed=0, device=dev, dtype=dtype)
        b = adrt.adrt(xt)
        M = precond.fit(n, h=4, samples=8, seed=0, device=dev, dtype=dtype) if op == "pcg" else None
        return (lambda: cgmod.cg(b, tol=1e-4, max_iters=200, graph=True, precond=M)), 0, batch
    if op == "precond":
        from adrt_gb300 import precond

        M = precond.ConvPreconditioner(sum(precond.basis(4)))
        return (lambda: M.apply(img)), es * batch * 2 * n * n, batch
    if op == "interp":
        from adrt_gb300 import utils

        return (lambda: utils.interp_to_cart(y)), es * batch * (A + 4 * n * n), batch
    if op == "unstitch":
        from adrt_gb300 import utils

        s = utils.stitch_adrt(y)
        return (lambda: utils.unstitch_adrt(s)), es * batch * 2 * A, batch
    if op == "coords":
        from adrt_gb300 import utils

        g = torch.Generator(device=dev)
        g.manual_seed(3)
        count = batch * n * n
        theta = (torch.rand(count, generator=g, device=dev, dtype=dtype) - 0.5) * 3.2
        tt = (torch.rand(count, generator=g, device=dev, dtype=dtype) - 0.5) * 1.4
        return (lambda: utils.coord_cart_to_adrt(theta, tt, n)), 0, batch
    if op in ("net_forward", "net_train"):
        from adrt_gb300.learned import PreconditionerNet

        net = PreconditionerNet(dev, seed=0)
        u = uniform_images(batch, n, seed=1, device=dev, dtype=torch.float32)
        if op == "net_forward":
            return (lambda: net.forward(u)), 0, batch
        t = uniform_images(batch, n, seed=2, device=dev, dtype=torch.float32)
        return (lambda: net.train_step(u, t, lr=1e-4)), 0, batch
    raise ValueError(f"unknown op {op}")


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--op", required=True, choices=OPS)
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--dtype", default="float32", choices=["float32", "float64"])
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--reps", type=int, default=5)
    a = ap.parse_args(argv)
    dev = torch.device("cuda", 0)
    dtype = torch.float32 if a.dtype == "float32" else torch.float64
    fn, nbytes, nimg = _setup(a.op, a.n, a.batch, dtype, dev)
    for _ in range(a.warmup):
        fn()
    s = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(a.reps):
        fn()
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.reps
    line = {"op": a.op, "n": a.n, "batch": a.batch, "dtype": a.dtype, "ms_per_call": ms,
            "img_s": nimg / (ms / 1e3)}
    if nbytes:
        line["algorithmic_gbs"] = nbytes / (ms / 1e3) / 1e9
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
