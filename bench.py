"""Benchmark of the VMC inner loop: walker-steps/s of (S MH steps + E_L).

One "step" is one request on a batch of walkers: ``S`` all-electron MH
updates followed by the forward-Laplacian local energy and its FP64 batch
mean/variance.  Default workload: FermiNet 4x(256, 32), K=16 on N2 (7+7
electrons), 4096 walkers, S=20 (the configuration the metric is quoted on).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(walkers are independent; no data-path collective) and rank 0 prints one
JSON line with the whole-job throughput.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "walker-steps/s (MH+E_L) mixed vs plain FP32 at |ΔĒ|≤0.5 mHa; serve p50/p99 ms"
UNIT = "walker-steps/s"
PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}

WORKLOADS = {
    "N2": dict(system="N2", nspins=(7, 7), walkers=4096, mh_steps=20),
    "Li": dict(system="Li", nspins=(2, 1), walkers=1024, mh_steps=10),
    "CH4": dict(system="CH4", nspins=(5, 5), walkers=4096, mh_steps=20),
    "C6H6": dict(system="C6H6", nspins=(21, 21), walkers=4096, mh_steps=10, model="psiformer"),
}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.tmp = None

    def start(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.tmp,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.tmp.flush()
        rows = []
        with open(self.tmp.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        load = [s for s in sm if mx and s >= 0.3 * max(mx)] or sm
        return {"sm_mhz": statistics.median(load) if load else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(
        os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(ms: float, device) -> float:
    """The slowest rank's time (every rank calls this after its timed region)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t)


def stream_layer_flops(cfg, n_atoms, B, T):
    """Algorithmic FLOPs of one launch set of the one-electron layer GEMMs for
    T tangent rows per electron: 2 * rows * (d_in + C*d2_in) * d_out summed over
    layers (the spin-mean term is a separate, per-walker GEMM)."""
    from jaqmc_gb300 import params as P
    C = cfg.channels
    tot = 0
    for (d1, d2, s, dd, upd) in P.FermiNetConfig.layer_dims(cfg, n_atoms):
        tot += 2 * B * cfg.n * T * (d1 + C * d2) * s
    return tot


# ----------------------------------------------------------------- CPU side
def cpu_request_rate(wl, seconds=12.0, sample_walkers=64, threads=None):
    """The oracle (torch FP32 on the host cores) running the same request on a
    bounded sample of walkers; returns (walker-steps/s, cores, description)."""
    import torch

    from jaqmc_gb300 import params as P
    from jaqmc_gb300 import systems as S
    from oracle import ferminet as OF
    from oracle import hamiltonian as OH
    threads = threads or os.cpu_count()
    torch.set_num_threads(threads)
    mol = S.SYSTEMS[wl["system"]]()
    cfg = P.FermiNetConfig(nspins=mol.nspins)
    tree = P.init_ferminet(cfg, mol.n_atoms, seed=0)
    oc = OF.FermiNetConfig(nspins=cfg.nspins, ndets=cfg.ndets)
    f = OF.logpsi_fn(tree, oc, mol.atoms, dtype=torch.float32)
    x = torch.as_tensor(S.init_walkers(mol, sample_walkers, seed=1))
    g = torch.Generator().manual_seed(2)
    S_ = wl["mh_steps"]
    reqs, t0 = 0, time.perf_counter()
    with torch.no_grad():
        while True:
            lp = 2 * f(x)
            for _ in range(S_):
                x2 = x + 0.02 * torch.randn(x.shape, generator=g)
                lp2 = 2 * f(x2)
                acc = (lp2 - lp) > torch.log(torch.rand(lp.shape, generator=g))
                x = torch.where(acc[:, None, None], x2, x)
                lp = torch.where(acc, lp2, lp)
            out = OF.evaluate(tree, oc, x, mol.atoms, dtype=torch.float32, tangents=True)
            el = OH.kinetic_from_tangents(out["grad"], out["lap"]) + OH.potential_energy(x, mol.atoms, mol.charges)
            float(el.double().mean())
            reqs += 1
            if time.perf_counter() - t0 >= seconds:
                break
    dt = time.perf_counter() - t0
    rate = reqs * sample_walkers * S_ / dt
    desc = (f"oracle (torch fp32, {threads} threads) on {sample_walkers} of {wl['walkers']} walkers, "
            f"{reqs} requests of {S_} MH steps + E_L in {dt:.1f} s")
    return rate, threads, desc


def cpu_psiformer_request_rate(seconds=12.0, sample_walkers=4, mh_steps=10, threads=None):
    """The oracle (torch FP32 on the host cores) running benzene Psiformer
    requests (``mh_steps`` MH updates + forward-Laplacian E_L) on a bounded
    sample of walkers; returns (walker-steps/s, cores, description)."""
    import torch

    from jaqmc_gb300 import params as P
    from jaqmc_gb300 import systems as S
    from oracle import hamiltonian as OH
    from oracle import psiformer as OP
    threads = threads or os.cpu_count()
    torch.set_num_threads(threads)
    mol = S.benzene()
    cfg = P.PsiformerConfig(nspins=mol.nspins)
    tree = P.init_psiformer(cfg, mol.n_atoms, seed=0)
    oc = OP.PsiformerConfig(nspins=cfg.nspins, ndets=cfg.ndets, num_layers=cfg.num_layers, num_heads=cfg.num_heads,
                            heads_dim=cfg.heads_dim, mlp_hidden_dims=list(cfg.mlp_hidden_dims),
                            envelope=cfg.envelope, orbitals_spin_split=cfg.orbitals_spin_split, jastrow=cfg.jastrow)
    f = OP.logpsi_fn(tree, oc, mol.atoms, dtype=torch.float32)
    x = torch.as_tensor(S.init_walkers(mol, sample_walkers, seed=1))
    g = torch.Generator().manual_seed(2)
    reqs, t0 = 0, time.perf_counter()
    with torch.no_grad():
        while True:
            lp = 2 * f(x)
            for _ in range(mh_steps):
                x2 = x + 0.02 * torch.randn(x.shape, generator=g)
                lp2 = 2 * f(x2)
                acc = (lp2 - lp) > torch.log(torch.rand(lp.shape, generator=g))
                x = torch.where(acc[:, None, None], x2, x)
                lp = torch.where(acc, lp2, lp)
            r = OP.evaluate_fl(tree, oc, x, mol.atoms, dtype=torch.float32)
            el = OH.kinetic_from_tangents(r["grad"], r["lap"]) + OH.potential_energy(x, mol.atoms, mol.charges)
            float(el.double().mean())
            reqs += 1
            if time.perf_counter() - t0 >= seconds:
                break
    dt = time.perf_counter() - t0
    rate = reqs * sample_walkers * mh_steps / dt
    desc = (f"oracle (torch fp32, {threads} threads) on {sample_walkers} walkers, "
            f"{reqs} requests of {mh_steps} MH steps + forward-Laplacian E_L in {dt:.1f} s")
    return rate, threads, desc


def run_reference(args, wl):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    rates = []
    psi = wl.get("model") == "psiformer"
    for _ in range(args.warmup):
        if psi:
            cpu_psiformer_request_rate(seconds=1.0, sample_walkers=2, mh_steps=wl["mh_steps"])
        else:
            cpu_request_rate(wl, seconds=1.0, sample_walkers=16)
    for _ in range(args.steps):
        if psi:
            r, cores, desc = cpu_psiformer_request_rate(seconds=4.0, sample_walkers=4, mh_steps=wl["mh_steps"])
        else:
            r, cores, desc = cpu_request_rate(wl, seconds=4.0, sample_walkers=32)
        rates.append(r)
    v = float(np.mean(rates))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": {"workload": workload_name(wl, "fp32"), **wl},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference (JAX/Flax) is not installable offline; its CPU path is timed as the "
                    "oracle restatement"}
    print(json.dumps(line), flush=True)
    return 0


def workload_name(wl, prec):
    if wl.get("model") == "psiformer":
        return (f"{wl['system']} Psiformer 4x(4x64), MLP 256, K=16, SimpleEE Jastrow, {wl['walkers']} walkers, "
                f"{wl['mh_steps']} MH steps + forward-Laplacian E_L, {prec}")
    return (f"{wl['system']} FermiNet 4x(256,32) K=16, {wl['walkers']} walkers, "
            f"{wl['mh_steps']} MH steps + forward-Laplacian E_L, {prec}")


# ----------------------------------------------------------------- Psiformer
def psiformer_forward_flops(cfg, n, A):
    """Dense FLOPs of one Psiformer log|psi| per walker: input layer, per layer
    QKV / output / MLP GEMMs and the two attention contractions, orbitals."""
    D, L = cfg.dim, cfg.num_layers
    mlp = list(cfg.mlp_hidden_dims) + [D]
    per_row = (4 * A + 1) * D
    layer = 3 * D * D + D * D
    din = D
    for dout in mlp:
        layer += din * dout
        din = dout
    per_row += L * layer + D * cfg.ndets * n
    attn = L * 2 * n * n * D
    return 2 * (n * per_row + attn)


def psiformer_attention_fl_roofline(cfg, n, walkers, attention_ms, prec="fp32"):
    """Roofline of the forward-Laplacian attention over one E_L of ``walkers``
    walkers: per (walker, head, layer) and per direction, the score tangents
    (2 n^2 Dh FMA), the cross term (n^2 Dh) and the mixing tangents with their
    cross term (3 n^2 Dh), over 3n directions: 18 n^3 Dh FMA.  FP32 form:
    k_psi_attention_fl against the measured FP32 SIMT peak.  Mixed form:
    k_attention_fl_mma issues three split-BF16 warp MMAs per product, so its
    achieved rate counts 3x the algorithmic FLOPs against the measured
    warp-MMA peak."""
    if not attention_ms:
        return None
    flop = 2.0 * 18 * n ** 3 * cfg.heads_dim * cfg.num_heads * cfg.num_layers * walkers
    t = attention_ms / 1e3
    if prec == "mixed" and MMA_PEAK["value"]:
        achieved = 3.0 * flop / t / 1e12
        peak = MMA_PEAK["value"]
        return {"kernel": "k_attention_fl_mma", "bound": "tensor (warp mma.sync, split BF16: 3 products)",
                "achieved": achieved, "peak": peak, "peak_kind": MMA_PEAK["source"], "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": None, "algorithmic_flop_per_request": flop,
                "algorithmic_tflops": flop / t / 1e12}
    achieved = flop / t / 1e12
    peak = SIMT_PEAK["value"]
    return {"kernel": "k_psi_attention_fl", "bound": "fp32 simt", "achieved": achieved, "peak": peak,
            "peak_kind": SIMT_PEAK["source"], "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
            "algorithmic_flop_per_request": flop}


def psiformer_request_roofline(cfg, n, A, walkers, mh_steps, ms, prec, pk, pk_kind):
    """Dense-tangent roofline of a whole request: (mh_steps + 3n + 2) forwards
    of psiformer_forward_flops per walker over the request's time, against the
    bf16 sustained peak (mixed form) or the FP32 SIMT peak (plain form)."""
    flop = psiformer_forward_flops(cfg, n, A) * (mh_steps + 3 * n + 2) * walkers
    achieved = flop / (ms / 1e3) / 1e12
    if prec == "mixed":
        peak, kind = pk["bf16_tflops_sustained"], f"bf16 sustained, {pk_kind}"
    else:
        peak, kind = SIMT_PEAK["value"], SIMT_PEAK["source"]
    return {"bound": "tensor" if prec == "mixed" else "fp32 simt", "achieved": achieved, "peak": peak,
            "peak_kind": kind, "unit": "TFLOP/s", "frac": achieved / peak, "algorithmic_tflop_per_request": flop / 1e12}


def run_psiformer(dev, steps, warmup, walkers=4096, mh_steps=10, oracle_walkers=32, burn_in=50,
                  forms=("mixed", "fp32")):
    """Benzene Psiformer (4 layers, 4 x 64 heads, MLP 256, K = 16, SimpleEE
    Jastrow): walker-steps/s of requests of ``mh_steps`` MH updates + the
    forward-Laplacian E_L and its FP64 mean/variance, in the split-BF16 and the
    FP32 form, on walkers burnt in from |psi|^2; the two forms' batch-mean
    energies on identical walkers, and both against the FP64 oracle on the
    first ``oracle_walkers`` walkers.  ``forms`` may name one form only (a
    profiler run); the cross-form figures are then left out."""
    import torch

    from jaqmc_gb300 import _native
    from jaqmc_gb300 import params as P
    from jaqmc_gb300 import systems as S
    mol = S.benzene()
    cfg = P.PsiformerConfig(nspins=mol.nspins)
    tree = P.init_psiformer(cfg, mol.n_atoms, seed=0)
    flat = torch.as_tensor(P.flatten(tree, P.psiformer_leaves(cfg, mol.n_atoms)), device=dev)
    models = {}
    for prec in forms:
        m = _native.NativePsiformer(cfg, mol.atoms, mol.charges, precision=prec, device=dev)
        m.set_params(flat)
        models[prec] = m
    x0 = torch.as_tensor(S.init_walkers(mol, walkers, seed=1), device=dev)
    models[forms[0]].mh_steps(x0, burn_in, 0.15, 1000, 0)

    def request(m, x, counter):
        m.mh_steps(x, mh_steps, 0.02, 2, counter)
        return _native.reduce_mean_var(m.local_energy(x)["e_local"])

    pk, pk_kind = peaks()
    names = {"stream_layer": "gemm", "pair": "attention", "means": "bias_act_residual_layernorm",
             "layer0": "input_layer", "orbital": "orbital", "logdet": "logdet", "features": "features_jastrow",
             "mh": "mh", "other": "other", "broadcast": "broadcast"}
    results = {}
    counter = 0
    for prec, m in models.items():
        x = x0.clone()
        for _ in range(warmup):
            request(m, x, counter)
            counter += mh_steps
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            mv = request(m, x, counter)
            counter += mh_steps
        e1.record()
        torch.cuda.synchronize()
        assert m.check_error() == 0
        ms = e0.elapsed_time(e1) / steps
        _native.profile_enable(True)
        _native.profile_read()
        request(m, x, counter)
        counter += mh_steps
        prof = _native.profile_read()
        _native.profile_enable(False)
        results[prec] = {"ms_per_request": ms, "walker_steps_per_s": walkers * mh_steps / (ms / 1e3),
                       "E_mean_var": mv.cpu().numpy().tolist(),
                       "gpu_launches_per_request": sum(v[0] for v in prof.values()),
                       "kernel_ms_per_request": {names.get(k, k): v[1] for k, v in prof.items() if v[0]},
                       "roofline_attention": psiformer_attention_fl_roofline(
                           cfg, mol.n_electrons, walkers, prof.get("pair", (0, 0.0))[1], prec),
                       "roofline_request": psiformer_request_roofline(
                           cfg, mol.n_electrons, mol.n_atoms, walkers, mh_steps, ms, prec, pk, pk_kind)}
    el = {p: m.local_energy(x0)["e_local"].double() for p, m in models.items()}
    d_mean = d_se = None
    if len(el) == 2:
        d = el["mixed"] - el["fp32"]
        d_mean = float(d.mean().abs())
        d_se = float(d.std() / d.numel() ** 0.5)
    d_oracle = None
    if oracle_walkers:
        from oracle import hamiltonian as OH
        from oracle import psiformer as OP
        sub = x0[:oracle_walkers].double().cpu()
        oc = OP.PsiformerConfig(nspins=cfg.nspins, ndets=cfg.ndets, num_layers=cfg.num_layers,
                                num_heads=cfg.num_heads, heads_dim=cfg.heads_dim,
                                mlp_hidden_dims=list(cfg.mlp_hidden_dims), envelope=cfg.envelope,
                                orbitals_spin_split=cfg.orbitals_spin_split, jastrow=cfg.jastrow)
        r = OP.evaluate_fl(tree, oc, sub, mol.atoms)
        el64 = (OH.kinetic_from_tangents(r["grad"], r["lap"]) + OH.potential_energy(sub, mol.atoms, mol.charges))
        d_oracle = {"walkers": int(sub.shape[0])}
        for p in models:
            d = (el[p][:oracle_walkers].cpu() - el64).numpy()
            ad = np.abs(d)
            d_oracle[p] = {"dE_mean_Ha": float(d.mean()), "paired_se_Ha": float(d.std(ddof=1) / np.sqrt(d.size)),
                           "median_abs_Ha": float(np.median(ad)), "max_abs_Ha": float(ad.max())}
    del models, el, x0, m, x, mv
    torch.cuda.empty_cache()  # the E_L workspaces (tens of GB) go back before the next leg
    cpu = None
    if oracle_walkers:
        r_, cores, desc = cpu_psiformer_request_rate(mh_steps=mh_steps)
        cpu = {"value": r_, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}
    return {"workload": f"C6H6 Psiformer 4x(4x64), MLP 256, K=16, SimpleEE Jastrow, {walkers} walkers, "
                        f"{mh_steps} MH steps + forward-Laplacian E_L",
            "walker_steps_per_s": results[forms[0]]["walker_steps_per_s"],
            "forms": results,
            "mixed_over_plain": (results["fp32"]["ms_per_request"] / results["mixed"]["ms_per_request"]
                                 if len(results) == 2 else None),
            "abs_dE_mean_mixed_vs_plain_Ha": d_mean,
            "dE_mean_paired_se_Ha": d_se,
            "dE_vs_fp64_oracle_Ha": d_oracle,
            "cpu_baseline": cpu}


# ---------------------------------------------------------------- gradient
def run_gradient(dev, steps, warmup, walkers=4096, budget_gb=8, burn_in=200, fd_walkers=2, fd_entries=64,
                 fd_step=1e-4):
    """The gradient path on CH4 (FermiNet 4 x (256, 32), K = 16, FP32): on
    ``walkers`` walkers burnt in from |psi|^2, with the adjoint's workspace
    budget set to ``budget_gb`` GiB (activations recomputed per chunk),
    (a) the per-walker Jacobian d log|psi_w| / d theta (B x P floats, caller
    buffer) and (b) the VMC energy gradient 2 <(E_L - E) d log|psi|>: E_L,
    its FP64 mean and one weighted adjoint pass.  Times per call by CUDA
    events; a check of the Jacobian against FP64 central differences of the
    oracle (step ``fd_step``) on ``fd_entries`` seeded entries for
    ``fd_walkers`` walkers of the same run."""
    import torch

    from jaqmc_gb300 import _native
    from jaqmc_gb300 import params as P
    from jaqmc_gb300 import systems as S
    mol = S.methane()
    cfg = P.FermiNetConfig(nspins=mol.nspins)
    tree = P.init_ferminet(cfg, mol.n_atoms, seed=0)
    leaves = P.ferminet_leaves(cfg, mol.n_atoms)
    flat_np = P.flatten(tree, leaves)
    m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, precision="fp32", device=dev)
    m.set_params(torch.as_tensor(flat_np, device=dev))
    m.set_grad_budget(budget_gb << 30)
    x = torch.as_tensor(S.init_walkers(mol, walkers, seed=1), device=dev)
    m.mh_steps(x, burn_in, 0.15, 1000, 0)
    Pn = m.param_count
    ws_bytes = m.lib.qmc_workspace_size(m.h, _native.OP_GRAD, walkers)
    # the adjoint runs in chunks of the largest batch whose workspace fits the
    # budget: the workspace stops growing at that batch
    lo, hi = 1, walkers
    while lo < hi:
        mid = (lo + hi) // 2
        if m.lib.qmc_workspace_size(m.h, _native.OP_GRAD, mid) >= ws_bytes:
            hi = mid
        else:
            lo = mid + 1
    chunk = lo
    J = torch.empty((walkers, Pn), dtype=torch.float32, device=dev)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    lp = torch.empty(walkers, dtype=torch.float32, device=dev)
    g = torch.empty(Pn, dtype=torch.float64, device=dev)
    stream = _native.stream_handle()

    def jac():
        _native.check(m.lib.qmc_grad(m.h, walkers, x.data_ptr(), None, J.data_ptr(), None, lp.data_ptr(),
                                     ws.data_ptr(), ws_bytes, stream))

    def vmc_grad():
        e = m.local_energy(x)["e_local"]
        mv = _native.reduce_mean_var(e)
        wts = (2.0 / walkers) * (e.double() - mv[0])
        _native.check(m.lib.qmc_grad(m.h, walkers, x.data_ptr(), wts.data_ptr(), None, g.data_ptr(),
                                     lp.data_ptr(), ws.data_ptr(), ws_bytes, stream))

    out = {}
    for name, fn in (("per_walker_jacobian", jac), ("vmc_energy_gradient", vmc_grad)):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        out[name] = {"ms_per_call": e0.elapsed_time(e1) / steps}
    assert m.check_error() == 0
    jb = walkers * Pn * 4
    out["per_walker_jacobian"].update({
        "jacobian_bytes": jb, "achieved_write_GBs": jb / (out["per_walker_jacobian"]["ms_per_call"] / 1e3) / 1e9})
    fd = None
    if fd_walkers:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from oracle import ferminet as OF
        xs = x[:fd_walkers].double().cpu()
        Jw = J[:fd_walkers].double().cpu().numpy()
        rng = np.random.default_rng(64)
        idx = rng.choice(Pn, fd_entries, replace=False)
        oc = OF.FermiNetConfig(nspins=cfg.nspins, ndets=cfg.ndets)
        base = flat_np.astype(np.float64)
        fdv = np.zeros((fd_walkers, fd_entries))
        for c, p in enumerate(idx):
            vals = []
            for sgn in (1.0, -1.0):
                v = base.copy()
                v[p] += sgn * fd_step
                tr = P.unflatten(v, leaves)
                vals.append(OF.evaluate(tr, oc, xs, mol.atoms, dtype=torch.float64)["logpsi"].numpy())
            fdv[:, c] = (vals[0] - vals[1]) / (2 * fd_step)
        scale = np.abs(Jw).max(axis=1, keepdims=True)
        fd = {"walkers": fd_walkers, "entries": fd_entries, "step": fd_step,
              "max_err_over_walker_scale": float((np.abs(Jw[:, idx] - fdv) / scale).max())}
    res = {"workload": f"CH4 FermiNet 4x(256,32) K=16 FP32, {walkers} walkers, adjoint budget {budget_gb} GiB",
           "params": Pn, "walkers": walkers, "workspace_bytes": int(ws_bytes),
           "walkers_per_chunk": chunk, "chunks": -(-walkers // chunk), **out, "fd_check": fd}
    del J, ws, m
    torch.cuda.empty_cache()
    return res


# ----------------------------------------------------------------- serving
def run_serving(dev, rate, n_jobs, requests, slots=8, seed=0, budget_gb=150, z_range=(2, 18),
                walker_choices=(256, 512, 1024, 2048, 4096), group_max=8):
    """Poisson(rate) arrivals of neutral-atom jobs (Z ~ U{z_range}, Hund
    spins, walkers ~ U{walker_choices}, parameters seed 0 so that jobs of one
    element share a model), each ``requests`` requests of 20 MH steps + E_L
    mean/variance in the mixed form, served with ``slots`` concurrent slots;
    queued requests of jobs sharing a model are packed into one launch set
    (up to ``group_max`` requests; 1: no packing)."""
    from jaqmc_gb300 import serving as SV
    be = SV.CudaBackend(precision="mixed", mh_steps=20, stddev=0.02, device=dev)
    warm = SV.Server(be, n_slots=2, hbm_budget=budget_gb << 30)
    warm.run_arrivals(SV.atom_job_specs(3, rate=0.0, seed=10_000, requests=2, walker_choices=(256,),
                                        z_range=z_range))
    srv = SV.Server(be, n_slots=slots, hbm_budget=budget_gb << 30, group_max=group_max)
    specs = SV.atom_job_specs(n_jobs, rate, seed=seed, requests=requests, z_range=z_range,
                              walker_choices=walker_choices)
    srv.run_arrivals(specs)
    first = min(sp.arrival for sp in specs)
    span = max(st.finished for st in srv.finished_jobs) - first
    lat, jl = srv.request_latencies_ms(), srv.job_latencies_ms()
    ws = sum(sp.walkers * 20 * requests for sp in specs)
    bad = [st.spec.job_id for st in srv.finished_jobs if not np.all(np.isfinite(np.stack(st.results)[:, :2]))]
    return {"arrival_rate_jobs_per_s": rate, "jobs": n_jobs, "requests_per_job": requests, "slots": slots,
            "elements_z": list(z_range), "walker_choices": list(walker_choices), "group_max": group_max,
            "hbm_budget_gb": budget_gb, "jobs_per_s": n_jobs / span, "requests_per_s": n_jobs * requests / span,
            "walker_steps_per_s": ws / span, "request_p50_ms": float(np.percentile(lat, 50)),
            "request_p99_ms": float(np.percentile(lat, 99)), "job_p50_ms": float(np.percentile(jl, 50)),
            "job_p99_ms": float(np.percentile(jl, 99)), "peak_hbm_gb": srv.peak_used / 1e9,
            "graph_replays": int(sum(r.graph for r in srv.finished)), "nonfinite_jobs": bad,
            "span_s": span, "packing": srv.packing()}


def run_request_only(args, wl):
    """W warm-up and K timed requests (or only their E_L / MH part) of one
    form, nothing else: the command line profiled by ncu."""
    import torch

    from jaqmc_gb300 import _native
    from jaqmc_gb300 import params as P
    from jaqmc_gb300 import systems as S
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    mol = S.SYSTEMS[wl["system"]]()
    if wl.get("model") == "psiformer":
        cfg = P.PsiformerConfig(nspins=mol.nspins)
        tree = P.init_psiformer(cfg, mol.n_atoms, seed=0)
        flat = torch.as_tensor(P.flatten(tree, P.psiformer_leaves(cfg, mol.n_atoms)), device=dev)
        m = _native.NativePsiformer(cfg, mol.atoms, mol.charges, precision=args.precision, device=dev)
    else:
        cfg = P.FermiNetConfig(nspins=mol.nspins)
        tree = P.init_ferminet(cfg, mol.n_atoms, seed=0)
        flat = torch.as_tensor(P.flatten(tree, P.ferminet_leaves(cfg, mol.n_atoms)), device=dev)
        m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, precision=args.precision, device=dev)
    B, S_ = wl["walkers"], wl["mh_steps"]
    x = torch.as_tensor(S.init_walkers(mol, B, seed=1), device=dev)
    m.set_params(flat)
    if args.burn_in:
        m.mh_steps(x, args.burn_in, 0.15, 1000, 0)

    def one(k):
        if args.op in ("request", "mh"):
            m.mh_steps(x, S_, 0.02, 2, k * S_)
        if args.op in ("request", "el"):
            _native.reduce_mean_var(m.local_energy(x)["e_local"])

    for k in range(args.warmup):
        one(k)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(args.steps):
        one(args.warmup + k)
    e1.record()
    torch.cuda.synchronize()
    assert m.check_error() == 0
    line = {"op": args.op, "precision": args.precision, "walkers": B, "system": wl["system"],
            "model": wl.get("model", "ferminet"),
            "ms_per_step": e0.elapsed_time(e1) / args.steps}
    if args.kernel_classes:
        _native.profile_enable(True)
        _native.profile_read()
        one(args.warmup + args.steps)
        prof = _native.profile_read()
        _native.profile_enable(False)
        line["kernel_ms"] = {k: round(v[1], 4) for k, v in prof.items() if v[0]}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- GPU side
def run_ours(args, wl):
    import torch
    import torch.distributed as dist

    from jaqmc_gb300 import _native
    from jaqmc_gb300 import params as P
    from jaqmc_gb300 import systems as S

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    measure_simt_peak(dev)
    mol = S.SYSTEMS[wl["system"]]()
    cfg = P.FermiNetConfig(nspins=mol.nspins)
    tree = P.init_ferminet(cfg, mol.n_atoms, seed=0)
    flat = torch.as_tensor(P.flatten(tree, P.ferminet_leaves(cfg, mol.n_atoms)), device=dev)
    B, S_ = wl["walkers"], wl["mh_steps"]
    x0 = torch.as_tensor(S.init_walkers(mol, B, seed=1 + rank), device=dev)
    models = {}
    for prec in ("fp32", "mixed"):
        m = _native.NativeFermiNet(cfg, mol.atoms, mol.charges, precision=prec, device=dev)
        m.set_params(flat)
        models[prec] = m
    stream = torch.cuda.current_stream()

    def request(m, x, counter):
        m.mh_steps(x, S_, 0.02, 2 + rank, counter)
        out = m.local_energy(x)
        return _native.reduce_mean_var(out["e_local"])

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(rg, K):
        # requests replayed from their CUDA graph on the timing stream
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(K):
            mv = rg.run(stream)
        e1.record(stream)
        barrier()
        return max_over_ranks(e0.elapsed_time(e1), dev), mv

    # burn-in: sample the walkers from |psi|^2 first (the reference's
    # SamplingWorkStage burn-in), so energies are those of a running VMC
    models["fp32"].mh_steps(x0, args.burn_in, 0.15, 1000 + rank, 0)
    torch.cuda.synchronize()
    prec_main = args.precision
    results = {}
    xs = {p: x0.clone() for p in models}
    counter = 0
    # each form's request captured once (after one eager run) and replayed
    graphs = {p: _native.RequestGraph(m, xs[p], S_, 0.02, 2 + rank, counter=1 << 20) for p, m in models.items()}
    for rg in graphs.values():
        for _ in range(args.warmup):
            rg.run()
    clocks = ClockSampler(local)
    clocks.start()
    for p in (prec_main,) + tuple(q for q in models if q != prec_main):
        ms, mv = timed(graphs[p], args.steps)
        results[p] = {"ms_per_step": ms / args.steps, "mean_var": mv.cpu().numpy().tolist()}
    clk = clocks.stop()

    # energy agreement of the two forms on identical walkers (same positions)
    xe = x0.clone()
    e_plain = models["fp32"].local_energy(xe)["e_local"].double()
    e_mixed = models["mixed"].local_energy(xe)["e_local"].double()
    d_mean = float((e_mixed.mean() - e_plain.mean()).abs())
    d_se = float((e_mixed - e_plain).std() / e_plain.numel() ** 0.5)
    d_oracle = None
    if rank == 0 and not args.no_cpu:
        d_oracle = oracle_energy_gap(models, tree, cfg, mol, xe[:args.oracle_walkers].contiguous())

    # live per-kernel timing of the same request (second pass, profiler on)
    _native.profile_enable(True)
    _native.profile_read()
    barrier()
    for k in range(args.steps):
        request(models[prec_main], xs[prec_main], counter + k * S_)
    barrier()
    prof = _native.profile_read()
    _native.profile_enable(False)
    launches = sum(v[0] for v in prof.values())

    # end to end through the public API with host buffers
    host_x = x0.cpu().pin_memory()
    host_out = torch.empty(2, dtype=torch.float64).pin_memory()
    rg = graphs[prec_main]
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.steps):
        rg.electrons.copy_(host_x, non_blocking=True)
        mv = rg.run(stream)
        host_out.copy_(mv, non_blocking=True)
    e1.record(stream)
    barrier()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, dev)

    ms_main = results[prec_main]["ms_per_step"]
    value = world * B * S_ / (ms_main / 1e3)
    value_e2e = world * B * S_ / (e2e_ms / 1e3)
    pk, pk_kind = peaks()
    # roofline of the dominant kernel: the one-electron layer kernel (layers
    # >= 1) in its forward-Laplacian launches, timed live on E_L-only passes
    _native.profile_enable(True)
    _native.profile_read()
    barrier()
    for _ in range(args.steps):
        models[prec_main].local_energy(xs[prec_main])
    barrier()
    prof_el = _native.profile_read()
    _native.profile_enable(False)
    Tp_fl = models[prec_main].tangent_rows(_native.OP_LOCAL_ENERGY)
    rl, rl_t = fl_layer_roofline(cfg, mol, B, Tp_fl, prec_main, prof_el, pk, pk_kind)
    psi = None
    if not args.no_psiformer:
        psi = run_psiformer(dev, max(1, args.steps // 2), 1)
    grad = None
    if not args.no_grad:
        grad = run_gradient(dev, max(1, args.steps // 2), 1, fd_walkers=0 if args.no_cpu else 2)
    serve = None
    if not args.no_serve:
        serve = {"by_arrival_rate": [run_serving(dev, float(r), args.serve_jobs, args.serve_requests,
                                                 slots=args.serve_slots) for r in args.serve_rates.split(",")],
                 # a burst of small jobs of one model (nitrogen atoms), served without and with
                 # packing of queued requests into one launch set
                 "same_model_burst": [run_serving(dev, 200.0, 64, 2, slots=args.serve_slots, seed=1,
                                                  z_range=(7, 7), walker_choices=(256, 512, 1024), group_max=g)
                                      for g in (1, 8)]}
    cpu = None
    if rank == 0 and not args.no_cpu:
        r, cores, desc = cpu_request_rate(wl)
        cpu = {"value": r, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}
    if rank == 0:
        # large nested blocks first, so that the end of the line (what a log
        # tail shows) carries the N2 figures
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_main, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16x3/fp32-acc" if prec_main == "mixed" else "fp32",
            "data": "synthetic (seeded walkers N(0,1) around nuclei; fan-in-scaled N(0,1/fan_in) params)",
            "config": {"workload": workload_name(wl, prec_main), **wl, "precision": prec_main,
                       "parallelism": f"replicas x{world}",
                       "launch": "each request replayed from one CUDA graph (RequestGraph)",
                       "l2": "working set larger than L2 (local-energy workspace several GB)"},
            "psiformer": psi,
            "gradient": grad,
            "serving": serve,
            "kernel_ms_per_step": {k: v[1] / args.steps for k, v in prof.items()},
            "gpu_launches": launches,
            "e2e": {"value": value_e2e, "unit": UNIT, "h2d_bytes_per_step": int(B * mol.n_electrons * 3 * 4),
                    "d2h_bytes_per_step": 16},
            "cpu_baseline": cpu,
            "clocks": clk,
            "fp32_simt_peak_tflops": SIMT_PEAK,
            "warp_mma_bf16_peak_tflops": MMA_PEAK,
            "roofline": rl,
            "roofline_tensor": rl_t,
            "roofline_request": {p_: ferminet_request_roofline(cfg, mol.n_atoms, world * B, S_, r_["ms_per_step"],
                                                               p_, pk, pk_kind) for p_, r_ in results.items()},
            "forms": {p_: {"ms_per_step": r_["ms_per_step"],
                           "walker_steps_per_s": world * B * S_ / (r_["ms_per_step"] / 1e3),
                           "E_mean_var": r_["mean_var"]} for p_, r_ in results.items()},
            "abs_dE_mean_mixed_vs_plain_Ha": d_mean,
            "dE_mean_paired_se_Ha": d_se,
            "dE_vs_fp64_oracle": d_oracle,
            "mixed_over_plain": results["fp32"]["ms_per_step"] / results["mixed"]["ms_per_step"],
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


# FP32 SIMT peak (TFLOP/s): measured on the device by the library's FMA probe
# (qmc_ffma_throughput) before the timed regions; the nominal figure
# (152 SMs x 128 FMA/clk x 2 FLOP x 2.07 GHz) stands only until then
SIMT_PEAK = {"value": 152 * 128 * 2 * 2.07e9 / 1e12, "source": "FP32 SIMT nominal (152 SM x 128 FMA x 2 x 2.07 GHz)"}


MMA_PEAK = {"value": None, "source": None}


def measure_simt_peak(dev):
    from jaqmc_gb300 import _native
    v = _native.fp32_simt_peak(dev)
    SIMT_PEAK.update(value=v, source="FP32 SIMT measured (FMA probe, CUDA events, best of 5)")
    MMA_PEAK.update(value=_native.warp_mma_peak(dev),
                    source="warp mma.sync BF16 measured (MMA probe, CUDA events, best of 5)")
    return v
# dram__bytes_read.sum + dram__bytes_write.sum of one forward-Laplacian launch
# of the one-electron layer kernel, from the committed ncu capture at 512
# walkers, scaled to the workload's walkers (traffic grows with the rows)
TRAFFIC_PER_WALKER: dict = {
    # ncu dram__bytes_read.sum + dram__bytes_write.sum of this launch at 512 walkers
    ("N2", "mixed"): (434.893056e6 + 283.123712e6) / 512,
}


def oracle_energy_gap(models, tree, cfg, mol, x, chunk=32):
    """Per form: the batch-mean E_L on ``x`` minus the FP64 oracle's, with the
    paired standard error of that difference (walker by walker), the median
    and maximum per-walker |dE_L| and the fraction within 1e-4 Ha."""
    import torch

    from oracle import ferminet as OF
    from oracle import hamiltonian as OH
    oc = OF.FermiNetConfig(nspins=cfg.nspins, ndets=cfg.ndets)
    el64 = []
    xc = x.double().cpu()
    for c0 in range(0, xc.shape[0], chunk):
        sub = xc[c0:c0 + chunk]
        ref = OF.evaluate(tree, oc, sub, mol.atoms, dtype=torch.float64, tangents=True)
        el64.append(OH.kinetic_from_tangents(ref["grad"], ref["lap"]) + OH.potential_energy(sub, mol.atoms,
                                                                                         mol.charges))
    el64 = torch.cat(el64).numpy()
    out = {"walkers": int(xc.shape[0])}
    for p_, m in models.items():
        d = m.local_energy(x)["e_local"].double().cpu().numpy() - el64
        ad = np.abs(d)
        out[p_] = {"dE_mean_Ha": float(d.mean()), "paired_se_Ha": float(d.std(ddof=1) / np.sqrt(d.size)),
                   "median_abs_Ha": float(np.median(ad)), "max_abs_Ha": float(ad.max()),
                   "frac_within_1e-4": float((ad <= 1e-4).mean())}
    return out


def ferminet_forward_flops(cfg, n_atoms):
    """Dense FLOPs of one FermiNet log|psi| forward per walker (2 per
    multiply-add): one-electron layers over [h1, spin means of h1 and h2]
    (src/jaqmc/wavefunction/backbone/ferminet.py:51-63), two-electron layers
    (:37-48) and the orbital projection to K x n orbitals per electron
    (src/jaqmc/wavefunction/output/orbital.py:60-78).  N2 at widths
    4 x (256, 32), K = 16: 20.58 MFLOP."""
    n, C = cfg.n, cfg.channels
    tot = 0
    for (d1, d2, s_, dd, upd) in cfg.layer_dims(n_atoms):
        tot += 2 * n * ((1 + C) * d1 + C * d2) * s_
        if upd:
            tot += 2 * n * n * d2 * dd
    tot += 2 * n * cfg.hidden_dims_single[-1] * cfg.ndets * n
    return tot


def ferminet_request_roofline(cfg, n_atoms, walkers, mh_steps, ms, prec, pk, pk_kind):
    """Dense-tangent roofline of a whole request: (mh_steps + 3n + 2) forwards
    of ferminet_forward_flops per walker over the request's time, against the
    bf16 sustained peak (mixed form) or the measured FP32 SIMT peak (plain)."""
    flop = ferminet_forward_flops(cfg, n_atoms) * (mh_steps + 3 * cfg.n + 2) * walkers
    achieved = flop / (ms / 1e3) / 1e12
    if prec == "mixed":
        peak, kind = pk["bf16_tflops_sustained"], f"bf16 sustained, {pk_kind}"
    else:
        peak, kind = SIMT_PEAK["value"], SIMT_PEAK["source"]
    return {"bound": "tensor" if prec == "mixed" else "fp32 simt", "achieved": achieved, "peak": peak,
            "peak_kind": kind, "unit": "TFLOP/s", "frac": achieved / peak,
            "algorithmic_tflop_per_request": flop / 1e12}


def fl_layer_bytes_flops(cfg, mol, B, Tp):
    """Algorithmic HBM bytes and FLOPs of one launch of a one-electron layer
    l >= 1 with Tp tangent rows per electron: activations in (k1), spin means
    of the pair stream (k2) and output (n_out) at 4 bytes per element (FP32,
    or hi+lo bf16), plus the per-walker broadcast term; FLOPs 2 rows k n_out."""
    from jaqmc_gb300 import params as P
    dims = P.FermiNetConfig.layer_dims(cfg, mol.n_atoms)
    d1_in, d2_in, d_out, _, _ = dims[1]
    k1, k2 = d1_in, cfg.channels * d2_in
    rows = B * mol.n_electrons * Tp
    nbytes = rows * (k1 + k2 + d_out) * 4 + B * Tp * d_out * 4
    flops = 2 * rows * (k1 + k2) * d_out
    return nbytes, flops


def fl_layer_roofline(cfg, mol, B, Tp, prec, prof_el, pk, pk_kind):
    launches, ms = prof_el["stream_layer"]
    if not launches:
        return None, None
    nbytes, flops = fl_layer_bytes_flops(cfg, mol, B, Tp)
    t = ms / launches / 1e3
    gbs = nbytes / t / 1e9
    kern = ("k_tc_gemm<EpiTcLayer>" if prec == "mixed" else "k_gemm_simt<EpiLayer<StF32>>")
    tpw = TRAFFIC_PER_WALKER.get((mol.name, prec))
    rl = {"kernel": f"{kern}: forward-Laplacian launch of a 256-wide layer, {B} walkers",
          "bound": "hbm", "achieved": gbs, "peak": pk["hbm_gbs"], "peak_source": f"hbm_gbs ({pk_kind})",
          "unit": "GB/s", "frac": gbs / pk["hbm_gbs"], "traffic": tpw * B if tpw else None,
          "algorithmic_bytes": nbytes, "ms_per_launch": t * 1e3, "launches": launches}
    if prec == "mixed":
        peak, src = pk["bf16_tflops_sustained"], f"bf16 dense sustained ({pk_kind})"
    else:
        peak, src = SIMT_PEAK["value"], SIMT_PEAK["source"]
    rl_t = {"bound": "tensor" if prec == "mixed" else "fp32-simt", "achieved": flops / t / 1e12, "peak": peak,
            "peak_source": src, "unit": "TFLOP/s", "frac": flops / t / 1e12 / peak, "algorithmic_flops": flops}
    return rl, rl_t


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="N2", choices=list(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["fp32", "mixed"])
    ap.add_argument("--burn-in", type=int, default=200)
    ap.add_argument("--oracle-walkers", type=int, default=256)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-psiformer", action="store_true")
    ap.add_argument("--no-grad", action="store_true", help="skip the CH4 gradient leg")
    ap.add_argument("--walkers", type=int, default=None, help="override the workload's walker count")
    ap.add_argument("--request-only", action="store_true",
                    help="only W warm-up + K timed requests of --precision (for profiler runs)")
    ap.add_argument("--op", default="request", choices=["request", "el", "mh"],
                    help="with --request-only: the whole request, only E_L, or only the MH steps")
    ap.add_argument("--kernel-classes", action="store_true",
                    help="with --request-only: add one profiled pass and its per-class kernel times")
    ap.add_argument("--serve-only", action="store_true", help="print only the serving measurement")
    ap.add_argument("--serve-rate", type=float, default=20.0, help="job arrival rate (jobs/s) of --serve-only")
    ap.add_argument("--serve-rates", default="10,40", help="arrival rates (jobs/s) of the serving leg")
    ap.add_argument("--serve-jobs", type=int, default=48)
    ap.add_argument("--serve-requests", type=int, default=2)
    ap.add_argument("--serve-slots", type=int, default=8)
    args = ap.parse_args()
    if args.serve_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(run_serving(torch.device("cuda", 0), args.serve_rate, args.serve_jobs,
                                     args.serve_requests, slots=args.serve_slots)), flush=True)
        return 0
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    wl = dict(WORKLOADS[args.workload])
    if args.walkers:
        wl["walkers"] = args.walkers
    if args.request_only:
        return run_request_only(args, wl)
    if wl.get("model") == "psiformer" and args.impl != "reference":
        import torch
        torch.cuda.set_device(0)
        measure_simt_peak(torch.device("cuda", 0))
        print(json.dumps(run_psiformer(torch.device("cuda", 0), args.steps, args.warmup, walkers=wl["walkers"],
                                       mh_steps=wl["mh_steps"], oracle_walkers=0 if args.no_cpu else 32)),
              flush=True)
        return 0
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_ours(args, wl)


if __name__ == "__main__":
    sys.exit(main())
