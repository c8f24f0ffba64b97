"""Benchmark of the GB300 LLG step: spin-steps/s of the stochastic Heun step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload: the large plain FP64 thermal run of the benchmark set, i.e. two-site cubic bcc 128^3
(4,194,304 spins), periodic, shells 8+6+12 with per-bond full 3x3 tensors (isotropic 20/10/-1 meV,
random symmetric anisotropic part at 1 %, random DMI |D| = 1 meV, J_ji = J_ij^T), uniaxial SIA
K = 0.01 meV, B = (0, 0, 0.5) T, T = 300 K, alpha = 0.05, dt = 0.1 fs, Philox noise.  Synthetic,
seeded; spins start uniform-random on the sphere.

One "step" = one Heun step of the whole lattice (predictor + corrector kernel).  `value` times K
steps with the spins resident in HBM (3 x 100 MB working set > 129 MB L2, so no L2 flush is needed);
`e2e` times K calls of the public drop-in API `GB300LLG.step(e_host)` with pinned host spins
(host->device copy, step, device->host copy per call).  Under torchrun each rank runs an
independent replica (weak scaling, no collective on the data path).

--impl reference times the reference's CPU algorithm (the C restatement of magex's fused numba
kernels in oracle/, all host threads, its own ziggurat noise) on the same workload.
"""
from __future__ import annotations

import argparse
import atexit
import datetime
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LLG spin-steps/s FP64 on 1×GB300 (%HBM roofline); batched vs plain; adjoint/fwd time"
UNIT = "spin-steps/s"
ALPHA, DT, TEMP, FIELD = 0.05, 1e-4, 300.0, (0.0, 0.0, 0.5)


def workload_config(L):
    return {"workload": f"bcc two-site {L}^3 ({2 * L ** 3:,} spins), 26 neighbours (8+6+12), full 3x3 tensors + DMI, "
                        f"SIA K=0.01 meV, B=(0,0,0.5) T, T=300 K, alpha=0.05, dt=0.1 fs, Philox noise, Heun",
            "spins": 2 * L ** 3, "neighbours": 26, "integrator": "heun", "noise": "philox",
            "l2": "inputs larger than L2 (3 x 24 B x N = 302 MB working set)", "parallelism": "replicas"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ------------------------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock / throttle samples (50 ms period, each with nvidia-smi's own timestamp).

    Started well before the timed region (nvidia-smi needs a few hundred ms to come up); `summary`
    keeps the samples whose timestamps fall between `mark_start` and `mark_end`.  A region shorter
    than the period may hold none: then the last sample before it and the first after it stand in,
    and the record says so (`window`)."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, index, period_ms=50):
        self.index, self.period_ms = index, period_ms
        self.proc, self.out, self.stopped = None, "", False
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        atexit.register(self.stop)          # never leave the sampler running after an error
        return self

    def mark_start(self):
        self.t0 = datetime.datetime.now()

    def mark_end(self):
        self.t1 = datetime.datetime.now()

    def stop(self):
        if self.proc is None or self.stopped:
            return
        self.stopped = True
        if self.proc.poll() is None:
            self.proc.terminate()
        try:
            self.out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            self.out, _ = self.proc.communicate()

    @classmethod
    def parse(cls, text):
        rows = []
        for line in text.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f")
                sm, smax = float(f[2]), float(f[3])
            except ValueError:
                continue
            rows.append((ts, sm, smax, {n for n, v in zip(cls.NAMES, f[6:10]) if v.lower() == "active"}))
        return rows

    def summary(self):
        if self.proc is None or self.t0 is None or self.t1 is None:
            return None
        rows = self.parse(self.out)
        inside = [r for r in rows if self.t0 <= r[0] <= self.t1]
        window = "timed region"
        if not inside:
            before = [r for r in rows if r[0] < self.t0]
            after = [r for r in rows if r[0] > self.t1]
            inside = before[-1:] + after[:1]
            window = f"bracketing samples (timed region shorter than the {self.period_ms} ms period)"
        if not inside:
            return None
        return {"sm_mhz": statistics.median(r[1] for r in inside), "sm_max_mhz": max(r[2] for r in inside),
                "reasons": sorted(set().union(*(r[3] for r in inside))), "samples": len(inside),
                "window": window, "period_ms": self.period_ms}


# ------------------------------------------------------------------------------------ CPU (oracle) timing
def cpu_oracle_timing(L, min_seconds=10.0, max_steps=400, steps=None, warmup=1):
    """The reference's CPU algorithm on the same workload: returns (spin-steps/s, steps, threads, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=L, field=FIELD)
    ora = oracle.OracleLLG(sc, ALPHA, DT, TEMP, seed=7, noise="ziggurat", csr="stencil", tuned=True)
    e = sc.init_spins("random", seed=1)
    for _ in range(warmup):
        ora.step_inplace(e)
    t0 = time.perf_counter()
    n = 0
    while True:
        ora.step_inplace(e)
        n += 1
        el = time.perf_counter() - t0
        if steps is not None:
            if n >= steps:
                break
        elif (el >= min_seconds and n >= 2) or n >= max_steps:
            break
    return sc.N * n / el, n, oracle.max_threads(), el


def cpu_flags():
    """Compiler flags of the timed CPU build (oracle/liboracle_tuned.so)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    return oracle.tuned_flags()


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    v, n, cores, el = cpu_oracle_timing(args.L, steps=args.steps, warmup=args.warmup)
    sample = (f"{n} Heun steps of the full {args.L}^3 two-site bcc lattice ({2 * args.L ** 3:,} spins), "
              f"C restatement of magex/fast.py _fused1/_fused2 with its ziggurat noise, OpenMP {cores} threads, "
              f"gcc {cpu_flags()}")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": n,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / n, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload_config(args.L),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------ GPU arm
def fp64_flops_per_spin_step(z):
    """Algorithmic FP64 flops of one Heun step per spin (FMA = 2): per stage 9 FMA per neighbour of the
    full-tensor gather (18 z), on-site gradient 18, field assembly 12, thermal add 6, LLG rhs 27,
    update + renormalisation 22 (predictor) / 25 (corrector)."""
    return 2 * 18 * z + 2 * (18 + 12 + 6 + 27) + 22 + 25


def read_ncu_traffic():
    """Per-launch DRAM bytes of the LLG kernels from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    out = {}
    if os.path.exists(path):
        for line in open(path):
            f = line.split()
            if len(f) >= 3 and f[1] == "bytes_per_launch_per_spin":
                out[f[0]] = float(f[2])
    return out


def bench_batched(K_batch=200, K_plain=20, nsys=256, log=None, precision="fp64"):
    """Uneven-film ensemble: 256 triangular films L in {32, 48, ..., 256}, J1 = 1 meV, interfacial DMI
    D/J = 0.3, K = 0.05 meV, B_z ~ U[0, 3] T, T ~ U[0, 20] K, alpha 0.1, dt 0.1 fs, Philox, seeded.
    Times the batched form (one persistent launch per stage, graph replays, autotuned launch shape)
    against per-system plain plans (one GB300LLG per film, each running its steps in one call)."""
    import torch
    from magex_gb300.batched import BatchedLLG
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import film_ensemble, triangle_list, triangular_film
    spec = film_ensemble(n=nsys, seed=0)
    films = [triangular_film(L=s["L"], field=s["B"]) for s in spec]
    Ts = [s["T"] for s in spec]
    seeds = list(range(1, nsys + 1))
    e0 = [sc.init_spins("random", seed=k) for k, sc in enumerate(films)]
    ens = BatchedLLG(films, 0.1, 1e-4, Ts, seeds, precision=precision)
    ens.set_spins(e0)
    ens.set_triangles([triangle_list(sc) for sc in films])
    best, timings = ens.autotune(steps=3)
    ntot = ens.ntot
    stream = torch.cuda.current_stream()
    ens.run(50, graph_chunk=50)                        # capture + warm-up
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    ens.run(K_batch, graph_chunk=50)
    b.record(stream)
    b.synchronize()
    t_batch = a.elapsed_time(b) * 1e-3
    rows = ens.rows()
    Q = ens.topological_charge()
    sols = [GB300LLG(sc, 0.1, 1e-4, Ts[k], seeds[k], precision=precision) for k, sc in enumerate(films)]
    lats = [sol.model.to_lattice(e0[k]) for k, sol in enumerate(sols)]
    for sol, lat in zip(sols, lats):
        sol.run_lattice(lat, 2)
    torch.cuda.synchronize()
    a.record(stream)
    for sol, lat in zip(sols, lats):
        sol.run_lattice(lat, K_plain)
    b.record(stream)
    b.synchronize()
    t_plain = a.elapsed_time(b) * 1e-3
    # the same per-system plans with their step loops replayed from CUDA graphs (runs of >= 64 steps of
    # lattices up to 2^21 sites); the graphs are captured in a first, untimed run
    K_graph = 64
    for sol, lat in zip(sols, lats):
        sol.run_lattice(lat, K_graph)
    torch.cuda.synchronize()
    a.record(stream)
    for sol, lat in zip(sols, lats):
        sol.run_lattice(lat, K_graph)
    b.record(stream)
    b.synchronize()
    t_graph = a.elapsed_time(b) * 1e-3
    v_batch = ntot * K_batch / t_batch
    v_plain = ntot * K_plain / t_plain
    v_graph = ntot * K_graph / t_graph
    return {"workload": f"{nsys} triangular films, L in {{32,48,...,256}} (uneven, {ntot:,} spins in total), "
                        "J1=1 meV, interfacial DMI D/J=0.3, K=0.05 meV, B_z~U[0,3] T, T~U[0,20] K, alpha 0.1, "
                        "dt 0.1 fs, Philox, FP64" + (" with the exact fixed-point exchange sum (batched and plain)"
                                                     if precision == "fp64_fixed" else ""),
            "value": v_batch, "unit": UNIT, "steps": K_batch, "plain_value": v_plain, "plain_steps": K_plain,
            "speedup_vs_plain": v_batch / v_plain, "plain_graph_value": v_graph, "plain_graph_steps": K_graph,
            "speedup_vs_plain_graphs": v_batch / v_graph, "launch": {"threads": best[0], "ctas_per_sm": best[1]},
            "autotune_ms_per_step": {f"{t}x{c}": round(v, 4) for (t, c), v in timings.items()},
            "ms_per_step": 1e3 * t_batch / K_batch, "gpu_launches_per_step": 2,
            "plain_gpu_launches_per_step": 2 * nsys,
            "final_mean_E_per_spin": float(np.mean(rows[:, 1])), "Q_range": [float(Q.min()), float(Q.max())]}


def bench_adjoint(L=128, nsteps=2000, seg=100, cache_bytes=0):
    """Differentiable-LLG workload: triangular 128 x 128, J1 = 1 meV, D/J = 0.3, K = 0.05 meV, B_z = 2 T,
    T = 0, alpha 0.3, dt 0.1 fs, 2000 Heun steps, checkpoint every 100 steps; loss = sum |e(T) - target|^2.
    Times the plain forward (GB300LLG), the checkpointed forward and the backward (recompute + adjoint)
    of magex_gb300.adjoint.llg_trajectory."""
    import torch
    from magex_gb300.adjoint import AdjointLLG, llg_trajectory
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import film_parameter_basis, triangular_film, uniaxial_sia
    sc = triangular_film(L=L, field=(0, 0, 2.0))
    adj = AdjointLLG(sc, alpha=0.3, dt=1e-4, seg_steps=seg, cache_bytes=cache_bytes)
    S_bond = film_parameter_basis(sc)
    S = torch.zeros((adj.groups.ngroups, 3, 3), dtype=torch.float64)
    for b in range(len(S_bond)):
        if not adj.groups.transposed[b]:
            S[adj.groups.group[b]] = torch.as_tensor(S_bond[b])
    e0 = sc.init_spins("random", seed=1)
    target = torch.as_tensor(sc.init_spins("random", seed=2), device=adj.device)
    plain = GB300LLG(sc, 0.3, 1e-4, 0.0, 1, precision="fp64")      # the all-FP64 forward
    default = GB300LLG(sc, 0.3, 1e-4, 0.0, 1)                      # the default solver ("auto")
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]

    def once(record):
        # gradients w.r.t. e(0), J1, D, K and B_z (the differentiable-LLG workload's parameters)
        theta = torch.tensor([1.0, 0.3, 0.05, 2.0], dtype=torch.float64, requires_grad=True)
        T = theta[0] * torch.eye(3, dtype=torch.float64)[None] + theta[1] * S
        zz = torch.zeros((3, 3), dtype=torch.float64)
        zz[2, 2] = 1.0
        A = (-theta[2] * (zz - torch.eye(3, dtype=torch.float64) / 3.0))[None]
        B = torch.stack([torch.zeros_like(theta[3]), torch.zeros_like(theta[3]), theta[3]])
        lat = plain.model.to_lattice(e0)
        e = torch.as_tensor(e0, device=adj.device).requires_grad_(True)
        torch.cuda.synchronize()
        if record:
            ev[0].record(stream)
        plain.run_lattice(lat, nsteps)
        if record:
            ev[1].record(stream)
        eT = llg_trajectory(adj, e, T, A, B, nsteps)
        loss = ((eT - target) ** 2).sum()
        if record:
            ev[2].record(stream)
        loss.backward()
        if record:
            ev[3].record(stream)
            lat2 = default.model.to_lattice(e0)
            ev[4].record(stream)
            default.run_lattice(lat2, nsteps)
            ev[5].record(stream)
        torch.cuda.synchronize()
        return theta.grad

    once(False)
    g = once(True)
    t_plain = ev[0].elapsed_time(ev[1])
    t_fwd = ev[1].elapsed_time(ev[2])
    t_bwd = ev[2].elapsed_time(ev[3])
    t_default = ev[4].elapsed_time(ev[5])
    return {"workload": f"triangular {L}x{L} film, J1=1 meV, D/J=0.3, K=0.05 meV, B_z=2 T, T=0, alpha 0.3, "
                        f"dt 0.1 fs, {nsteps} Heun steps, checkpoint every {seg}, loss sum|e(T)-target|^2, FP64",
            "cache_bytes": cache_bytes,
            "resident_segments": min(len(adj._segments(nsteps)), adj._cache_budget() // (8 * adj.storage_doubles)),
            "forward_plain_ms": t_plain, "forward_checkpointed_ms": t_fwd, "backward_ms": t_bwd,
            "adjoint_over_forward": t_bwd / t_plain, "gradient_total_over_forward": (t_fwd + t_bwd) / t_plain,
            "default_forward": {"precision": default.precision, "ms": t_default,
                                "adjoint_over_forward": t_bwd / t_default},
            "grad_J1_D_K_Bz": [float(x) for x in g]}


def bench_config5(nsys=64, L=64, K=10, adj_steps=1000, seed=0, precision="fp64"):
    """Large batched + adjoint workload: nsys two-site bcc L^3 systems (524,288 spins each at L = 64),
    4 shells (8+6+12+24) with one seeded full 3x3 tensor per shell (iso 20/10/-1/1 meV, 1% anisotropic,
    DMI 5% of |J|), transposed on reverse bonds, SIA K = 0.01 meV, B = (0, 0, 0.5) T, T ~ U[0, 600] K,
    alpha 0.05, dt 0.1 fs, Philox, FP64.  Times K steps of the batched form against per-system plain
    plans, then the adjoint of the mean-energy loss w.r.t. the 4 shell tensors on one system at 300 K
    over adj_steps steps, with the checkpointed segments kept in HBM as far as the free memory allows."""
    import torch
    from magex_gb300.adjoint import AdjointLLG, CouplingGroups, energy_per_site, llg_trajectory
    from magex_gb300.batched import BatchedLLG
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site, uniaxial_sia
    rng = np.random.default_rng(seed)
    Ts = [float(t) for t in rng.uniform(0.0, 600.0, nsys)]
    sc = bcc_two_site(L=L, J=(20.0, 10.0, -1.0, 1.0), dmi_frac=0.05, per="shell", seed=1, field=FIELD)
    stream = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ens = BatchedLLG([sc] * nsys, ALPHA, DT, Ts, list(range(1, nsys + 1)), precision=precision)
    ens.set_spins([sc.init_spins("random", seed=k) for k in range(nsys)])
    ens.run(2, graph_chunk=2)
    torch.cuda.synchronize()
    a.record(stream)
    ens.run(K, graph_chunk=K)
    b.record(stream)
    b.synchronize()
    t_batch = a.elapsed_time(b) * 1e-3
    rows = ens.rows()
    del ens
    sols = [GB300LLG(sc, ALPHA, DT, Ts[k], 1 + k, precision=precision) for k in range(nsys)]
    lats = [sol.model.to_lattice(sc.init_spins("random", seed=k)) for k, sol in enumerate(sols)]
    for sol, lat in zip(sols, lats):
        sol.run_lattice(lat, 1)
    torch.cuda.synchronize()
    a.record(stream)
    for sol, lat in zip(sols, lats):
        sol.run_lattice(lat, K)
    b.record(stream)
    b.synchronize()
    t_plain = a.elapsed_time(b) * 1e-3
    del sols, lats
    torch.cuda.empty_cache()
    ntot = nsys * sc.N
    head = {"workload": f"{nsys} two-site bcc {L}^3 systems ({ntot:,} spins), 4 shells 8+6+12+24 with seeded "
                        "per-shell full 3x3 tensors (iso 20/10/-1/1 meV, 1% anisotropic, DMI 5%), K=0.01 meV, "
                        "B=(0,0,0.5) T, T~U[0,600] K, alpha 0.05, dt 0.1 fs, Philox, FP64" +
                        (" with the exact fixed-point exchange sum" if precision == "fp64_fixed" else ""),
            "batched_value": ntot * K / t_batch, "plain_value": ntot * K / t_plain, "unit": UNIT, "steps": K,
            "speedup_vs_plain": t_plain / t_batch, "batched_ms_per_step": 1e3 * t_batch / K,
            "final_mean_E_per_spin": float(np.mean(rows[:, 1]))}
    if adj_steps <= 0:
        return head

    groups = CouplingGroups.per_shell(sc)
    free, _ = torch.cuda.mem_get_info()
    cache = int(0.6 * free)
    adj = AdjointLLG(sc, groups, alpha=ALPHA, dt=DT, temperature=300.0, seed=77, seg_steps=100, cache_bytes=cache)
    plain = GB300LLG(sc, ALPHA, DT, 300.0, 77, precision="fp64")     # the all-FP64 forward
    default = GB300LLG(sc, ALPHA, DT, 300.0, 77)                      # the default solver ("auto")
    A0 = torch.as_tensor(np.stack([uniaxial_sia(0.01)] * sc.ns))
    B0 = torch.tensor(FIELD, dtype=torch.float64)
    e0 = torch.as_tensor(sc.init_spins("random", seed=5), device=adj.device)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(7)]

    def once(record):
        T = torch.as_tensor(adj.T0).clone().requires_grad_(True)
        lat = plain.model.to_lattice(e0)
        torch.cuda.synchronize()
        if record:
            ev[0].record(stream)
        plain.run_lattice(lat, adj_steps)
        if record:
            ev[1].record(stream)
        eT = llg_trajectory(adj, e0, T, A0, B0, adj_steps)
        if record:
            ev[2].record(stream)
        loss = energy_per_site(sc, groups, eT, T, A0, B0).mean()
        if record:
            ev[3].record(stream)
        loss.backward()
        if record:
            ev[4].record(stream)
            lat2 = default.model.to_lattice(e0)
            ev[5].record(stream)
            default.run_lattice(lat2, adj_steps)
            ev[6].record(stream)
        torch.cuda.synchronize()
        return float(loss.detach()), T.grad

    once(False)
    loss, g = once(True)
    t = [ev[0].elapsed_time(ev[k]) for k in range(1, 5)]
    t_default = ev[5].elapsed_time(ev[6])
    return {**head,
            "adjoint": {"system": f"one {L}^3 system ({sc.N:,} spins) at 300 K", "steps": adj_steps,
                        "loss": "mean energy per spin after the trajectory (meV)",
                        "parameters": "4 shell tensors (36 entries), canonical and transposed bonds",
                        "resident_segments": len(adj._segments(adj_steps)), "cache_bytes": cache,
                        "forward_plain_ms": t[0], "forward_checkpointed_ms": t[1] - t[0],
                        "loss_ms": t[2] - t[1], "backward_ms": t[3] - t[2],
                        "adjoint_over_forward": (t[3] - t[2]) / t[0], "loss_value": loss,
                        "forward_precision": adj.precision,
                        "default_forward": {"precision": default.precision, "ms": t_default,
                                            "adjoint_over_forward": (t[3] - t[2]) / t_default},
                        "grad_norm_per_shell": [float(x) for x in g.reshape(4, -1).norm(dim=1)]}}


def bench_mc_points(sizes=(8, 16), npts=16, therm=1000, meas=4000):
    """Monte Carlo T scan of magex's mc workflow (the input of a T_c estimate): npts temperatures for
    each sc L^3 ferromagnet size (J = 1 meV), therm + meas sweeps each (Gaussian moves +
    over-relaxation, sigma adapted every 50 sweeps, E and the order vector sampled every 5 sweeps):
    wall time of points() (one ensemble per size, the sizes on concurrent streams) against the points
    run one by one with point() (magex runs each point as its own process, magex/montecarlo.py:390-401)."""
    import numpy as np
    from magex_gb300.mc import point, points
    from magex_gb300.spinmodel import load_results, make_model
    uc = load_results(make_model("sc", J=[1.0]))
    c = dict(sigma=0.6, overrelax=1, move="gaussian", init="random", init_axis=(0.0, 0.0, 1.0),
             therm_sweeps=therm, meas_sweeps=meas, sample_every=5)
    Ts = np.linspace(10.0, 40.0, npts)
    jobs = [(uc, (L, L, L), (True,) * 3, (0.0, 0.0, 0.0), float(T), c, 100 + i)
            for L in sizes for i, T in enumerate(Ts)]
    point(jobs[0])
    t_one = {}
    for L in sizes:
        job = next(j for j in jobs if j[1][0] == L)
        t0 = time.perf_counter()
        one = point(job)
        t_one[L] = time.perf_counter() - t0
    t0 = time.perf_counter()
    rows = points(jobs)
    t_all = time.perf_counter() - t0
    assert rows[-npts]["E"] == one["E"]
    spins = sum(L ** 3 for L in sizes) * npts
    seq = sum(t_one[L] * npts for L in sizes)
    return {"workload": f"sc L^3 for L in {list(sizes)}, {npts} temperatures 10..40 K each, {therm} + {meas} sweeps, "
                        "Gaussian moves + 1 over-relaxation pass, Philox, FP64",
            "points_s": t_all, "one_point_s": {str(L): t_one[L] for L in sizes},
            "speedup_vs_points_one_by_one": seq / t_all,
            "site_updates_per_s": 2 * spins * (therm + meas) / t_all, "unit": "site-updates/s",
            "rows_equal_point": True}


def bench_mc_pt(L=16, nrep=16, therm=1000, meas=4000):
    """Parallel tempering (magex/advanced_mc.py:38-95): nrep replicas of an sc L^3 ferromagnet on
    30..45 K, therm + meas sweeps, swaps every 5 sweeps, samples every 2: wall time and swap
    acceptance."""
    import numpy as np
    from magex_gb300.lattice import Supercell
    from magex_gb300.mc import parallel_tempering
    from magex_gb300.spinmodel import load_results, make_model
    sc = Supercell(load_results(make_model("sc", J=[1.0])), (L, L, L), (True,) * 3, (0.0, 0.0, 0.0))
    Ts = np.linspace(30.0, 45.0, nrep)
    parallel_tempering(sc, Ts, therm_sweeps=50, meas_sweeps=50)
    t0 = time.perf_counter()
    rows, swap = parallel_tempering(sc, Ts, therm_sweeps=therm, meas_sweeps=meas, sample_every=2, swap_every=5)
    t = time.perf_counter() - t0
    return {"workload": f"parallel tempering, sc {L}^3, {nrep} replicas on 30..45 K, {therm} + {meas} sweeps, "
                        "swaps every 5 sweeps, Gaussian moves + 1 over-relaxation pass, Philox, FP64",
            "seconds": t, "site_updates_per_s": 2 * sc.N * nrep * (therm + meas) / t, "unit": "site-updates/s",
            "swap_acceptance": [round(x, 3) for x in swap]}


def bench_mc(L=128, sweeps=20, move="gaussian", overrelax=1, cpu_baseline=True, precision="fp64"):
    """Monte Carlo colour sweeps on the 128^3 two-site bcc workload (4,194,304 spins, z = 26, full
    3x3 tensors), T = 300 K, in-kernel Philox draws: site updates per second (one update = one trial
    move or one over-relaxation reflection of one spin)."""
    import torch
    from magex_gb300.mc import MetropolisMC
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=L, field=FIELD)
    mc = MetropolisMC(sc, TEMP, seed=1, sigma=0.3, overrelax=overrelax, move=move, precision=precision)
    lat = mc.model.to_lattice(sc.init_spins("random", seed=1))
    mc.sweep_lattice(lat, 3)
    mc.acceptance()
    stream = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    mc.sweep_lattice(lat, sweeps)
    b.record(stream)
    b.synchronize()
    t = a.elapsed_time(b) * 1e-3
    ncol = mc.ncolors
    updates = sc.N * (1 + overrelax) * sweeps
    acc = mc.acceptance()
    del mc, lat
    cpu = None
    if cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        from oracle import OracleMC, max_threads
        ora = OracleMC(sc, TEMP, 1, 0.3, overrelax, move, csr="stencil")
        e = sc.init_spins("random", seed=1)
        ora.sweep(e)
        n, t0 = 0, time.perf_counter()
        while n < 2 or (time.perf_counter() - t0 < 10.0 and n < 10):
            ora.sweep(e)
            n += 1
        el = time.perf_counter() - t0
        cpu = {"value": sc.N * (1 + overrelax) * n / el, "unit": "site-updates/s", "cores": max_threads(),
               "kind": "port", "sample": f"{n} sweeps of the same lattice, {el:.1f} s: C restatement of magex's "
                                         "NumPy colour sweep (OpenMP over each class) with magex's NumPy draws"}
    return {"workload": f"two-site bcc {L}^3 ({sc.N:,} spins), T = 300 K, {move} moves + {overrelax} over-relaxation "
                        "pass per sweep, Philox, FP64" + (" with the exact fixed-point exchange sum"
                                                          if precision == "fp64_fixed" else ""),
            "value": updates / t, "unit": "site-updates/s", "sweeps": sweeps, "ms_per_sweep": 1e3 * t / sweeps,
            "colour_classes": ncol, "acceptance": acc, "gpu_launches_per_sweep": ncol * (1 + overrelax),
            "cpu_baseline": cpu}


def bench_sqw(L=128, reps=20):
    """S(q, w) sampling cost on the 128^3 two-site bcc lattice: one device Fourier projection of the
    spins onto a Gamma-X-M-Gamma-R path of commensurate wave vectors (every point at L resolution)."""
    import torch
    from magex_gb300.device import DeviceModel
    from magex_gb300.spectra import FourierProjector
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=L, field=FIELD)
    dm = DeviceModel(sc)
    h = L // 2
    G, X, M, R = np.zeros(3), np.array([0.5, 0, 0]), np.array([0.5, 0.5, 0]), np.array([0.5, 0.5, 0.5])
    pts = []
    for a, b in ((G, X), (X, M), (M, G), (G, R)):
        for k in range(h):
            pts.append(a + (b - a) * k / h)
    q = np.round(np.array(pts) * L) / L
    proj = FourierProjector(dm, q)
    lat = dm.to_lattice(sc.init_spins("random", seed=1))
    out = proj.project(lat)
    stream = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(reps):
        proj.project(lat, out=out)
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b) / reps
    return {"workload": f"two-site bcc {L}^3 ({sc.N:,} spins), {len(q)} wave vectors on Gamma-X-M-Gamma-R",
            "ms_per_sample": ms, "hbm_gbs": 24.0 * sc.N / (ms * 1e-3) / 1e9,
            "note": "one pass over e (24 B per spin) plus O(nq ns L^2) work; magex's dense phase matrix for this "
                    f"case would hold {16 * sc.N * len(q) / 1e9:.0f} GB"}


def bench_texture(L=256, reps=20):
    """Topological charge of a triangular L x L film through magex_gb300.texture (the drop-in for
    magex/texture.py:30-63): the first call builds and keeps the periodic Delaunay triangulation,
    later calls are one device pass over the triangles.  magex repeats the triangulation and the
    NumPy solid-angle sum on every call; both are timed here on the host beside the device call."""
    import time
    import torch
    from magex_gb300 import texture
    from magex_gb300.workloads import triangular_film
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import solid_angle_charge
    sc = triangular_film(L=L, field=(0, 0, 0))
    e = torch.as_tensor(sc.init_spins("random", seed=3), device="cuda")
    t0 = time.perf_counter()
    tri, sign = texture.layer_triangles(sc)
    t_tri = time.perf_counter() - t0
    texture.topological_charge(sc, e)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        Q = texture.topological_charge(sc, e)
    t_dev = (time.perf_counter() - t0) / reps
    e_host = e.cpu().numpy()
    t0 = time.perf_counter()
    Q_host = solid_angle_charge(e_host, tri, sign)
    t_sum = time.perf_counter() - t0
    return {"workload": f"triangular {L} x {L} film ({sc.N:,} spins, {len(tri):,} triangles), random spins",
            "ms_per_call": t_dev * 1e3, "host_triangulation_ms": t_tri * 1e3, "host_solid_angle_sum_ms": t_sum * 1e3,
            "abs_diff_vs_host": abs(Q - Q_host),
            "note": "ms_per_call is the wall time of texture.topological_charge on a device tensor after the first "
                    "call (which also triangulates); magex pays triangulation + sum on every call"}


def bench_callers(L=128, fmr_steps=20000, relax_L=64, cpu_steps=400):
    """Two callers of the step on a triangular film (J = 1 meV, D = 0.3 meV interfacial, K = 0.05
    meV, mu = 2 mu_B, B_z = 1 T): the FMR ring-down of magex/programs.py:124-150 (L x L, fmr_steps
    steps, a sample every 5 steps) and the damped-LLG relaxation of magex/minimize.py:168-181 from
    random spins (relax_L x relax_L, tol 1e-4 meV).  Wall time of the whole call; beside each, the
    oracle's step loop on the host cores for cpu_steps steps of the same system."""
    import torch
    from magex_gb300.minimize import minimize
    from magex_gb300.programs import fmr
    from magex_gb300.workloads import triangular_film
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import OracleLLG, max_threads

    def cpu_rate(sc, alpha, dt, precession):
        ora = OracleLLG(sc, alpha, dt, 0.0, precession=precession, csr="stencil", tuned=True)
        e = sc.init_spins("random", seed=2)
        t0 = time.perf_counter()
        for _ in range(cpu_steps):
            ora.step_inplace(e)
        return sc.N * cpu_steps / (time.perf_counter() - t0)

    out = {}
    sc = triangular_film(L=L, field=(0, 0, 1.0))
    e0 = sc.init_spins("ferro", (0, 0, 1))
    fmr(sc, e0, steps=200)                                   # warm-up (graphs, buffers)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, fpk, table = fmr(sc, e0, steps=fmr_steps)
    el = time.perf_counter() - t0
    out["fmr"] = {"workload": f"triangular {L} x {L} film ({sc.N:,} spins), {fmr_steps} steps, a sample every 5",
                  "seconds": el, "value": sc.N * fmr_steps / el, "unit": UNIT, "f_peak_GHz": fpk,
                  "cpu_baseline": {"value": cpu_rate(sc, 0.001, 2e-3, True), "unit": UNIT, "cores": max_threads(),
                                   "kind": "port", "sample": f"{cpu_steps} oracle steps of the same film"}}
    sc = triangular_film(L=relax_L, field=(0, 0, 1.0))
    e0 = sc.init_spins("random", seed=5)
    minimize(sc, e0, "llg", tol=1e-4, max_iter=200)        # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, info = minimize(sc, e0, "llg", tol=1e-4)
    el = time.perf_counter() - t0
    out["relax"] = {"workload": f"triangular {relax_L} x {relax_L} film ({sc.N:,} spins) from random spins, "
                                "tol 1e-4 meV",
                    "iterations": info["iterations"], "seconds": el, "value": sc.N * info["iterations"] / el,
                    "unit": UNIT,
                    "cpu_baseline": {"value": cpu_rate(sc, 1.0, 2e-3, False), "unit": UNIT, "cores": max_threads(),
                                     "kind": "port", "sample": f"{cpu_steps} oracle steps of the same film"}}
    return out


def bench_onsite_higher(L=128, steps=50):
    """The headline step with magex's cubic (Kc = 0.02 meV, axes along x, y, z) and higher uniaxial
    (K2 = 0.01, K3 = 0.005 meV along z) anisotropy on every site: the EXTRA kernels that evaluate them
    beside the plain ones, on the same two-site bcc L^3 lattice."""
    import torch
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=L, field=FIELD)
    sc.cubic = (np.full(sc.N, 0.02), np.eye(3))
    sc.uniaxial_higher = (np.full(sc.N, 0.01), np.full(sc.N, 0.005), np.array([0.0, 0.0, 1.0]))
    sol = GB300LLG(sc, ALPHA, DT, TEMP, 3)
    lat = sol.model.to_lattice(sc.init_spins("random", seed=1))
    sol.run_lattice(lat, 3)
    stream = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    sol.run_lattice(lat, steps)
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b) / steps
    return {"workload": f"two-site bcc {L}^3 ({sc.N:,} spins) with cubic and higher uniaxial anisotropy on every site",
            "value": sc.N / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "steps": steps}


def bench_config1(steps=1000, cpu=True):
    """Plain FP64 workload of the reference's CPU-runnable case: simple-cubic 16^3 (4,096 spins), 6
    neighbours, J = 1 meV, mu = 2 mu_B, alpha 0.1, B = 0, T = 0, dt 0.1 fs, 1000 Heun steps from
    random spins.  Small enough that launches dominate: run_lattice replays CUDA graphs of 32 steps."""
    import torch
    from magex_gb300.lattice import Supercell
    from magex_gb300.llg import GB300LLG
    from magex_gb300.spinmodel import load_results, make_model
    sc = Supercell(load_results(make_model("sc", a=3.0, J=[1.0], moment=2.0)), (16, 16, 16))
    e0 = sc.init_spins("random", seed=1)
    out = {"workload": "sc 16^3 (4,096 spins), J = 1 meV, alpha 0.1, T = 0, dt 0.1 fs, 1000 Heun steps, FP64",
           "unit": UNIT, "steps": steps}
    for prec in ("fp64", "fp64_fixed"):
        sol = GB300LLG(sc, 0.1, 1e-4, 0.0, 1, precision=prec)
        lat = sol.model.to_lattice(e0)
        sol.run_lattice(lat, 64)
        stream = torch.cuda.current_stream()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        sol.run_lattice(lat, steps)
        b.record(stream)
        b.synchronize()
        ms = a.elapsed_time(b)
        out[prec] = {"value": sc.N * steps / (ms * 1e-3), "ms_total": ms, "us_per_step": 1e3 * ms / steps}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        from oracle import OracleLLG, max_threads
        ora = OracleLLG(sc, 0.1, 1e-4, 0.0, 1, csr="stencil", tuned=True)
        e = e0.copy()
        t0 = time.perf_counter()
        for _ in range(steps):
            ora.step_inplace(e)
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": sc.N * steps / el, "unit": UNIT, "cores": max_threads(), "kind": "port",
                               "sample": f"the full {steps} steps, {el:.2f} s"}
    return out


def bench_reduced(L, K, warmup, precision):
    """The same workload with a reduced-FP64 step form: precision="df32" (exchange gather on compensated
    FP32 pairs) or "int48" (exchange gather in exact 48-bit fixed-point integer arithmetic); both keep
    the spins, the integration and the renormalisation FP64 and evaluate the rest of the field and the
    right-hand side on FP32 pairs.  Reported beside the FP64 value, never as it."""
    import torch
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    sc = bcc_two_site(L=L, field=FIELD)
    e0 = sc.init_spins("random", seed=1)
    sols = {p: GB300LLG(sc, ALPHA, DT, TEMP, seed=1000, precision=p) for p in ("fp64", precision)}
    lat = {p: sols[p].model.to_lattice(e0) for p in sols}
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        sols[precision].run_lattice(lat[precision], 1)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    sols[precision].run_lattice(lat[precision], K)
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b) / K
    # same Philox stream through the FP64 plan: the deviation after warmup + K steps
    sols["fp64"].run_lattice(lat["fp64"], warmup + K)
    torch.cuda.synchronize()
    dev = float((lat["fp64"] - lat[precision]).abs().max())
    what = {"df32": "exchange gather on compensated FP32 pairs (~44 bits)",
            "int48": "exchange gather as exact integer arithmetic on 48-bit fixed point (INT32 pipe)",
            "fp64_fixed": "exchange and on-site sums exact on 56-bit fixed point (INT32 pipe); every "
                          "floating-point operation FP64"}[precision]
    # algorithmic bytes per spin-step: predictor e, split in; ep, k1, split out; corrector split, k1, e in; e, split out
    split = 8
    nbytes = (24 + split + 24 + 24 + 3 * split) + (3 * split + 24 + 24 + 24 + 3 * split) - split
    tail = ("" if precision == "fp64_fixed" else
            "; integration and renormalisation FP64, field remainder and right-hand side on FP32 pairs")
    return {"precision": what + tail,
            "value": sc.N / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "steps": K,
            "max_abs_deviation_from_fp64_plan": dev, "deviation_after_steps": warmup + K,
            "algorithmic_bytes_per_spin_step": nbytes,
            "hbm_roofline_frac": nbytes * sc.N / (ms * 1e-3) / 1e9 / 6760.6}

def _r(x, n=4):
    return None if x is None else float(f"{x:.{n}g}")


def bench_fp64_plan(sc, e0, K, warmup, peak64, flops_step, hbm_peak):
    """The all-FP64 plan (precision="fp64") on the same workload: K steps through mgx_llg_run, its
    per-kernel times and both roofline fractions (HBM at 72 / 96 B per site; FP64 pipe at
    flops_step per spin-step against the live-measured DFMA peak)."""
    import torch
    from magex_gb300.llg import GB300LLG
    sol = GB300LLG(sc, ALPHA, DT, TEMP, seed=3000, precision="fp64")
    lat = sol.model.to_lattice(e0)
    stream = torch.cuda.current_stream()
    sol.run_lattice(lat, warmup)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    torch.cuda.synchronize()
    ev[0].record(stream)
    sol.stage_lattice(lat, 0)
    ev[1].record(stream)
    sol.stage_lattice(lat, 1)
    ev[2].record(stream)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    sol.run_lattice(lat, K)
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b) / K
    pm, cm = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    N = sc.N
    return {"value": N / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "steps": K,
            "kernels_ms": {"k_predict": pm, "k_correct": cm},
            "hbm_roofline_frac": 96.0 * N / (cm * 1e-3) / 1e9 / hbm_peak,
            "fp64_roofline": {"achieved": flops_step * N / (ms * 1e-3) / 1e12, "peak": peak64 / 1e12,
                              "unit": "TFLOP/s", "frac": flops_step * N / (ms * 1e-3) / peak64,
                              "flops_per_spin_step": flops_step,
                              "peak_source": "measured live (mgx_measure_fp64_peak, DFMA loop)"}}


def north_star_summary(line):
    """The figures the benchmark targets grade, compact: spin-steps/s and roofline fractions of the
    FP64 step and of its exact fixed-point-sum form, batched / per-system speed-ups, adjoint / forward
    time ratios (recompute and resident), and the large batched + adjoint workload."""
    fp = line["fp64_plan"]
    out = {"default": {"precision": line["config"]["precision"], "value": _r(line["value"]),
                       "hbm_frac": _r(line["roofline"]["frac"], 3)},
           "fp64": {"value": _r(fp["value"]), "hbm_frac": _r(fp["hbm_roofline_frac"], 3),
                    "fp64_pipe_frac": _r(fp["fp64_roofline"]["frac"], 3)}}
    fx = line.get("fp64_fixed_gather_variant")
    if fx:
        out["fp64_fixed_dev_vs_fp64"] = _r(fx["max_abs_deviation_from_fp64_plan"], 2)
    for key in ("batched", "batched_fp64_fixed"):
        b = line.get(key)
        if b:
            out[key] = {"value": _r(b["value"]), "speedup_vs_plain": _r(b["speedup_vs_plain"], 3),
                        "speedup_vs_plain_graphs": _r(b["speedup_vs_plain_graphs"], 3)}
    for key in ("adjoint", "adjoint_resident", "adjoint_large"):
        a = line.get(key)
        if a:
            out[key + "_bwd_over_fwd"] = _r(a["adjoint_over_forward"], 3)
            d = a.get("default_forward")
            if d and d["precision"] != "fp64":
                out[key + "_bwd_over_default_fwd"] = _r(d["adjoint_over_forward"], 3)
    c5 = line.get("large_batched_adjoint")
    if c5:
        a5 = c5.get("adjoint", {})
        out["config5"] = {"batched_value": _r(c5["batched_value"]), "speedup_vs_plain": _r(c5["speedup_vs_plain"], 3),
                          "adjoint_bwd_over_fwd": _r(a5.get("adjoint_over_forward"), 3),
                          "adjoint_bwd_over_default_fwd": _r(a5.get("default_forward", {}).get("adjoint_over_forward"), 3)}
    c5f = line.get("large_batched_fp64_fixed")
    if c5f:
        out["config5_fp64_fixed"] = {"batched_value": _r(c5f["batched_value"]),
                                     "speedup_vs_plain": _r(c5f["speedup_vs_plain"], 3)}
    out["e2e"] = _r(line["e2e"]["value"])
    if "cpu_baseline" in line:
        out["cpu_baseline"] = _r(line["cpu_baseline"]["value"])
    return out


def run_gb300(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from magex_gb300 import _lib, build
    build.build_library()
    from magex_gb300.llg import GB300LLG
    from magex_gb300.workloads import bcc_two_site
    import ctypes as C

    lib = _lib.load()
    clk = ClockSampler(local).start()   # running well before the timed region
    peak64 = C.c_double()
    _lib.check(lib.mgx_measure_fp64_peak(C.byref(peak64)), "fp64 peak")

    sc = bcc_two_site(L=args.L, field=FIELD)
    N = sc.N
    z = len(sc.bond_src) / sc.ns
    e0 = sc.init_spins("random", seed=1 + rank)
    # the default solver: precision "auto" is the FP64 step with the exact fixed-point exchange sum
    # for this model (every floating-point operation FP64)
    sol = GB300LLG(sc, ALPHA, DT, TEMP, seed=1000 + rank)
    prec = sol.precision
    lat = sol.model.to_lattice(e0)
    stream = torch.cuda.current_stream()
    sol.run_lattice(lat, args.warmup)
    K = args.steps
    # per-kernel durations: CUDA events around each stage call on the launching stream (the stage-0
    # call of a fixed-point plan also refreshes the fixed-point copy of the spins: one split kernel)
    Kk = min(K, 50)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * Kk + 1)]
    torch.cuda.synchronize()
    ev[0].record(stream)
    for k in range(Kk):
        sol.stage_lattice(lat, 0)
        ev[2 * k + 1].record(stream)
        sol.stage_lattice(lat, 1)
        ev[2 * k + 2].record(stream)
    torch.cuda.synchronize()
    pred_ms = [ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(Kk)]
    corr_ms = [ev[2 * k + 1].elapsed_time(ev[2 * k + 2]) for k in range(Kk)]
    # the timed region: K steps through one public call (mgx_llg_run)
    a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clk.mark_start()
    a_ev.record(stream)
    sol.run_lattice(lat, K)
    b_ev.record(stream)
    torch.cuda.synchronize()
    clk.mark_end()
    if ws > 1:
        dist.barrier()
    clk.stop()
    total_ms = a_ev.elapsed_time(b_ev)
    norm_err = float((torch.linalg.vector_norm(lat, dim=0) - 1).abs().max())
    if not (norm_err < 1e-12):
        raise RuntimeError(f"spins lost unit norm during the benchmark: {norm_err}")

    # end to end through the public API with pinned host buffers
    e_host = torch.from_numpy(e0).pin_memory()
    out_host = torch.empty_like(e_host).pin_memory()
    sol2 = GB300LLG(sc, ALPHA, DT, TEMP, seed=2000 + rank)
    # warm-up over both (input, output) buffer pairs the timed loop alternates between (each pair's
    # slab pipeline is captured as a graph on its first call)
    cur = e_host
    for _ in range(2 * max(2, args.warmup // 2)):
        sol2.step(cur, out=out_host)
        cur, out_host = out_host, cur
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(K):
        sol2.step(cur, out=out_host)
        cur, out_host = out_host, cur
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0

    from magex_gb300.replicas import max_over_ranks
    total_ms, e2e_s = max_over_ranks([total_ms, e2e_s], dist if ws > 1 else None)
    if rank != 0:
        dist.destroy_process_group()
        return

    value = N * K * ws / (total_ms * 1e-3)
    pm, cm = statistics.mean(pred_ms), statistics.mean(corr_ms)
    fixed = prec == "fp64_fixed"
    names = ("k_fx_split + k_predict_fx", "k_correct_fx") if fixed else ("k_predict", "k_correct")
    dominant, dom_ms = (names[1], cm) if cm >= pm else (names[0], pm)
    # algorithmic HBM bytes per site.  FP64 plan: predictor reads e, writes ep, k1 (72); corrector reads
    # ep, k1, e, writes e (96).  Fixed-point plan: the split reads e and writes its 56-bit copy es (48);
    # the predictor reads e, es and writes ep, k1 and the copy eps (120); the corrector reads eps, k1,
    # ep, e and writes e, es (144).  Neighbour rows come from L1 / L2 (the stencil re-reads them).
    bytes_per_spin = {"k_predict": 72.0, "k_correct": 96.0, "k_fx_split + k_predict_fx": 168.0,
                      "k_correct_fx": 144.0}[dominant]
    hbm_peak = None
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        hbm_peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    else:
        hbm_peak, peak_src = 6800.0, "fallback"
    achieved = bytes_per_spin * N / (dom_ms * 1e-3) / 1e9
    # measured DRAM bytes per spin of every kernel of the timed pair (the split and the predictor for
    # the fixed-point plan), None unless all of them were captured
    per_kernel = read_ncu_traffic()
    parts = [per_kernel.get(k) for k in dominant.split(" + ")]
    traffic = None if any(v is None for v in parts) else sum(parts)
    flops_step = fp64_flops_per_spin_step(z)
    clocks = clk.summary()
    # the all-FP64 plan on the same workload, beside the default
    plain = bench_fp64_plan(sc, e0, min(K, 200), args.warmup, peak64.value, flops_step, hbm_peak)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": args.warmup,
        "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded two-site bcc model, random initial spins)",
        "config": {**workload_config(args.L), "precision": prec,
                   "arithmetic": ("every floating-point operation FP64; exchange and on-site sums exact on 56-bit "
                                  "fixed-point spins and couplings (INT32 pipe), rounded once" if fixed else
                                  "all FP64")},
        "gpu_launches": 2 * K + (1 if fixed else 0),
    }
    # secondary measurements first (bulky), the graded figures last: a reader of the line's tail sees
    # the roofline, the CPU baseline, e2e and the compact spec summary
    if ws == 1 and not args.no_batched:
        line["monte_carlo"] = bench_mc(L=args.L, cpu_baseline=not args.no_cpu_baseline)
        line["monte_carlo_fp64_fixed"] = bench_mc(L=args.L, cpu_baseline=False, precision="fp64_fixed")
        line["monte_carlo_points"] = bench_mc_points()
        line["monte_carlo_parallel_tempering"] = bench_mc_pt()
        line["sqw_projection"] = bench_sqw(L=args.L)
        line["topological_charge"] = bench_texture()
        line["callers"] = bench_callers()
        line["onsite_higher"] = bench_onsite_higher()
    if ws == 1:
        line["config1_sc16"] = bench_config1(cpu=not args.no_cpu_baseline)
        line["df32_gather_variant"] = bench_reduced(args.L, min(K, 200), args.warmup, "df32")
        line["int48_gather_variant"] = bench_reduced(args.L, min(K, 200), args.warmup, "int48")
        line["fp64_fixed_gather_variant"] = bench_reduced(args.L, min(K, 200), args.warmup, "fp64_fixed")
    if ws == 1 and not args.no_batched and not args.no_adjoint:
        line["large_batched_adjoint"] = bench_config5()
        line["large_batched_fp64_fixed"] = bench_config5(precision="fp64_fixed", adj_steps=0)
    if ws == 1 and not args.no_batched:
        line["batched"] = bench_batched()
        line["batched_fp64_fixed"] = bench_batched(precision="fp64_fixed")
    if ws == 1 and not args.no_adjoint:
        line["adjoint"] = bench_adjoint()
        # the same trajectory with the default checkpoint policy: segments resident in up to half the
        # free HBM (2000 steps x 14 N doubles = 3.7 GB here), so nothing is recomputed
        line["adjoint_resident"] = bench_adjoint(cache_bytes="auto")
        line["adjoint_large"] = bench_adjoint(L=1024, nsteps=200, seg=50)
    line["kernels_ms"] = {names[0]: pm, names[1]: cm}
    line["fp64_plan"] = plain
    if ws == 1 and not args.no_cpu_baseline:
        v, n, cores, el = cpu_oracle_timing(args.L)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"{n} Heun steps of the full {args.L}^3 lattice ({N:,} spins), {el:.1f} s, "
                                          "C restatement of magex's fused numba kernels + ziggurat noise "
                                          f"(OpenMP {cores} threads, gcc {cpu_flags()})"}
    line["e2e"] = {"value": N * K * ws / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 24 * N,
                   "d2h_bytes_per_step": 24 * N,
                   "api": "GB300LLG.step(pinned host (N,3) float64) -> pinned host (N,3): one mgx_llg_step_host "
                          "call, copies in axis-0 slabs overlapping the stages"}
    line["roofline"] = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                        "frac": achieved / hbm_peak, "peak_source": peak_src,
                        "traffic": None if traffic is None else traffic * N,
                        "traffic_source": "profiles/ncu_traffic.txt (ncu dram bytes per spin of this kernel x N)",
                        "algorithmic_bytes_per_launch": bytes_per_spin * N, "launch_ms": dom_ms}
    line["clocks"] = clocks
    line["north_star"] = north_star_summary(line)
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--L", type=int, default=128, help="bcc cells per side (default: the 128^3 workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint / forward timing")
    ap.add_argument("--only", choices=["adjoint", "batched", "df32", "int48", "fp64_fixed", "config1", "config5", "mc",
                                       "sqw", "texture", "callers", "onsite_higher"],
                    default=None,
                    help="run only one of the secondary measurements and print its JSON (for profiling)")
    ap.add_argument("--adjoint-steps", type=int, default=None)
    ap.add_argument("--adjoint-L", type=int, default=128)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.only:
        import torch
        torch.cuda.set_device(0)
        from magex_gb300 import build
        build.build_library()
        if args.only == "adjoint":
            out = bench_adjoint(L=args.adjoint_L, nsteps=args.adjoint_steps or 2000)
        elif args.only in ("df32", "int48", "fp64_fixed"):
            out = bench_reduced(args.L, args.steps, args.warmup, args.only)
        elif args.only == "config1":
            out = bench_config1()
        elif args.only == "sqw":
            out = bench_sqw(L=args.L)
        elif args.only == "texture":
            out = bench_texture()
        elif args.only == "callers":
            out = bench_callers()
        elif args.only == "onsite_higher":
            out = bench_onsite_higher()
        elif args.only == "mc":
            out = [bench_mc(L=args.L, sweeps=min(args.steps, 100), cpu_baseline=False, precision=p)
                   for p in ("fp64", "fp64_fixed")]
            if args.steps >= 20:           # short profiling runs skip the T scan's ~300k launches
                out += [bench_mc_points(), bench_mc_pt()]
        elif args.only == "config5":
            out = [bench_config5(K=min(args.steps, 50), adj_steps=args.adjoint_steps or 1000),
                   bench_config5(K=min(args.steps, 50), adj_steps=0, precision="fp64_fixed")]
        else:
            out = [bench_batched(), bench_batched(precision="fp64_fixed")]
        print(json.dumps(out), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
