#!/usr/bin/env python
"""Benchmark of the GB300 pruning likelihood.

One step = one whole-tree evaluation of the b3 pruning likelihood (every
internal dirty, as after ``mark_all_edges_updated``) on a synthetic workload
with the shape of the largest configuration: 256 taxa, 20,000 DNA sites
simulated under GTR + Gamma4 (exchangeabilities ~ Gamma(2,1), frequencies ~
Dirichlet(5,5,5,5), alpha 0.5) on a Yule tree of root height 1.0, in the
chosen form (FP32 partials, power-of-two rescaling, FP64 site sum).

Metric: pruning GB/s = algorithmic bytes of one evaluation (a closed formula
over the dirty list, see aspartik_gb300/schedule.py) / time.
  value     K back-to-back evaluations, device time between CUDA events on
            the calculator's stream; the alignment, partials and model are
            resident; each step still uploads its dirty list and lengths.
  e2e       the same steps through the public C ABI with host buffers: every
            step copies its dirty list and edge lengths host->device, runs,
            and reads the log-likelihood back (blocking), host-timed.
  roofline  the pruning kernel alone (per-launch CUDA events) against the
            measured HBM copy bandwidth.

``--impl reference`` times the reference's CPU pruner (the C restatement of
crates/b3/src/calculator/cpu4.rs, all host threads) on the same workload and
prints the same metric computed with the same byte count, so the ratio of the
two arms is the ratio of evaluations per second.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from aspartik_gb300 import schedule, sim  # noqa: E402

METRIC = "pruning GB/s (whole-tree evaluation, chosen FP32 form)"
UNIT = "GB/s"

WORKLOADS = {
    # largest configuration: 256 taxa, 20,000 sites, GTR + Gamma4
    "dna256x20000_gtr_g4": dict(taxa=256, sites=20000, model="gtr", alpha=0.5, categories=4,
                                root_height=1.0, pi_conc=5.0),
    # 64 taxa, 10,000 sites, GTR + Gamma4
    "dna64x10000_gtr_g4": dict(taxa=64, sites=10000, model="gtr", alpha=0.5, categories=4,
                               root_height=1.0, pi_conc=5.0),
    # 16 taxa, 1,000 sites, HKY(kappa 2), one category
    "dna16x1000_hky": dict(taxa=16, sites=1000, model="hky", alpha=None, categories=1,
                           root_height=0.5, pi_conc=10.0),
}
DEFAULT_WORKLOAD = "dna256x20000_gtr_g4"
# DRAM bytes (read + write) of one whole-tree launch of prune4_runs_kernel on
# the default workload, from an ncu capture (dram__bytes_read.sum 17.47 MB +
# dram__bytes_write.sum 304.28 MB): children written earlier in the same pass
# are read from shared-memory slots or from L2, tables are built on chip, so
# the traffic is mostly the partials' writes, 43 % of the algorithmic bytes.
TRAFFIC_RUNS_BYTES = 321_756_416


def make_workload(name: str, seed: int = 4) -> dict:
    spec = WORKLOADS[name]
    rng = np.random.default_rng(seed)
    tree = sim.yule_tree(spec["taxa"], rng, root_height=spec["root_height"])
    pi = sim.dirichlet([spec["pi_conc"]] * 4, rng)
    rates = sim.hky_rates(2.0) if spec["model"] == "hky" else rng.gamma(2.0, 1.0, size=6)
    Q = sim.reversible_q(rates, pi)
    K = spec["categories"]
    cats = sim.gamma_rates(spec["alpha"], K) if spec["alpha"] else np.ones(1)
    states = sim.simulate_alignment(tree, spec["sites"], Q, pi, rng, cat_rates=cats)
    leaves, weights, _ = sim.deduplicate(sim.to_dna_codes(states))
    return dict(spec=spec, tree=tree, pi=pi, rates=rates, cats=cats, leaves=leaves,
                weights=weights, top=schedule.Topology(tree.parents, tree.heights))


# ---------------------------------------------------------------------------
# clocks during the timed region


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------


T_START = time.perf_counter()


def progress(what: str) -> None:
    """One line per finished leg on stderr (the JSON line stays alone on
    stdout)."""
    print(f"[bench {time.perf_counter() - T_START:7.1f} s] {what}", file=sys.stderr, flush=True)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allreduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def make_calc(wl, precision: str, device: int):
    from aspartik_gb300.calculator import Calculator

    K = wl["spec"]["categories"]
    calc = Calculator.GB300(device, precision).make4(wl["leaves"], wl["leaves"].shape[1],
                                                     num_categories=K)
    calc.set_weights(wl["weights"])
    calc.set_reversible(wl["rates"], wl["pi"])
    if wl["spec"]["alpha"]:
        calc.set_gamma(wl["spec"]["alpha"])
    return calc


def device_throughput(calc, lists, steps, warmup, world):
    """Device time of `steps` back-to-back evaluations (no per-launch
    events, as a caller runs them), then the same evaluations again with
    CUDA events around each kernel for the per-kernel times."""
    internals, children, lengths = lists
    calc.set_timing(False)
    for _ in range(warmup):
        calc.propose_lengths(internals, children, lengths, 1.0)
    calc.log_likelihood()
    barrier(world)
    calc.span_begin()
    for _ in range(steps):
        calc.propose_lengths(internals, children, lengths, 1.0)
    ms = calc.span_end()
    barrier(world)
    calc.set_timing(True)
    calc.timing_totals(reset=True)
    for _ in range(steps):
        calc.propose_lengths(internals, children, lengths, 1.0)
    calc.log_likelihood()
    tt, tp, n = calc.timing_totals(reset=True)
    calc.set_timing(False)
    return ms, tt / max(n, 1), tp / max(n, 1), n


class CpuReference:
    """The restated cpu4 on (a pattern sample of) the workload, built once:
    one calculator per category as GammaLikelihood runs them
    (likelihood/gamma.rs:97-169), the transition matrices of the whole tree,
    `threads` host threads.  `evaluate()` times one whole-tree evaluation
    (propose of every category, log-sum-exp mixing, weighted sum)."""

    def __init__(self, wl, num_threads: int, pattern_limit: int | None = None):
        from oracle import oracle as O

        leaves, weights = wl["leaves"], wl["weights"]
        if pattern_limit is not None and pattern_limit < leaves.shape[1]:
            leaves = np.ascontiguousarray(leaves[:, :pattern_limit])
            weights = weights[:pattern_limit]
        self.P = leaves.shape[1]
        self.weights = weights.astype(np.float64)
        self.pi = wl["pi"]
        self.internals, self.children, lengths = wl["top"].full()
        model = O.gtr(wl["rates"], wl["pi"])
        cats = O.gamma_categories(wl["spec"]["alpha"], wl["spec"]["categories"]) \
            if wl["spec"]["alpha"] else np.ones(1)
        self.mats = [np.stack([model.transition(d * r) for d in lengths.reshape(-1)])
                     for r in cats]
        self.calcs = [O.Cpu4Calculator(leaves, self.P, 30, num_threads) for _ in cats]
        self.threads = self.calcs[0].num_threads()

    def evaluate(self):
        """One evaluation, accepted: every propose is followed by an accept,
        as the reference's call order requires (two proposals in one epoch
        would double-count its scale sums, cpu4.rs:403-433)."""
        t0 = time.perf_counter()
        per = []
        for calc, m in zip(self.calcs, self.mats):
            calc.propose(self.internals, self.children, m, self.pi)
            per.append(calc.likelihoods())
            calc.accept()
        per = np.array(per)
        mx = per.max(axis=0)
        site = mx + np.log(np.exp(per - mx).sum(axis=0)) + np.log(1.0 / len(self.calcs))
        lnl = float(site @ self.weights)
        return time.perf_counter() - t0, lnl


def batched(device: int, steps: int, warmup: int, chains: int = 32, seed: int = 4) -> dict:
    """Many chains in one launch: `chains` calculators with taxa uniform on
    24..200 and sites log-uniform on 500..50,000 (i.i.d. random bases, as
    Msa::random), GTR+Gamma4, each step one CUDA-graph replay evaluating every
    chain.  Reports whole-tree evaluations (all chains, aggregate algorithmic
    GB/s) and dirty-path evaluations (a random node's path in every chain)."""
    from aspartik_gb300.calculator import Batch, Calculator

    rng = np.random.default_rng(seed)
    members, tops, whole = [], [], []
    total_bytes, patterns = 0, 0
    for _ in range(chains):
        L = int(rng.integers(24, 201))
        N = int(np.exp(rng.uniform(np.log(500), np.log(50000))))
        tree = sim.yule_tree(L, rng, root_height=1.0)
        leaves, weights, _ = sim.deduplicate(sim.random_dna(L, N, rng))
        pi = sim.dirichlet([5.0] * 4, rng)
        calc = Calculator.GB300(device, "f32").make4(leaves, leaves.shape[1], num_categories=4)
        calc.set_weights(weights)
        calc.set_reversible(rng.gamma(2.0, 1.0, size=6), pi)
        calc.set_gamma(0.5)
        top = schedule.Topology(tree.parents, tree.heights)
        members.append(calc)
        tops.append(top)
        whole.append(top.full())
        P = leaves.shape[1]
        patterns += P
        total_bytes += schedule.algorithmic_bytes(top, whole[-1][0], P, 4, 4, w=4, e_b=4, w_p=4)
    batch = Batch(members)

    def step(lists):
        for calc, lst in zip(members, lists):
            calc.stage_lengths(*lst, 1.0)
        batch.run()
        return batch.log_likelihoods()

    for _ in range(warmup):
        step(whole)
    dev_ms = 0.0
    t0 = time.perf_counter()
    for _ in range(steps):
        lnl = step(whole)
        dev_ms += batch.last_ms()
    wall = time.perf_counter() - t0
    # dirty paths
    paths = [[top.path(int(v)) for v in rng.integers(top.L, 2 * top.L - 1, size=8)]
             for top in tops]
    dsteps = max(steps, 50)
    for k in range(warmup):
        step([p[k % 8] for p in paths])
    t0 = time.perf_counter()
    dms = 0.0
    for k in range(dsteps):
        step([p[k % 8] for p in paths])
        dms += batch.last_ms()
    dwall = time.perf_counter() - t0
    batch.close()
    for m in members:
        m.close()
    return {"chains": chains, "patterns_total": patterns, "categories": 4,
            "whole_tree": {"value": round(steps * total_bytes / (dev_ms * 1e-3) / 1e9, 2),
                           "unit": "GB/s", "device_ms_per_step": round(dev_ms / steps, 4),
                           "wall_ms_per_step": round(wall * 1e3 / steps, 4),
                           "bytes_per_step": total_bytes,
                           "finite": bool(np.isfinite(lnl).all())},
            "dirty_path": {"device_us_per_step": round(dms * 1e3 / dsteps, 2),
                           "wall_us_per_step": round(dwall * 1e6 / dsteps, 2),
                           "chain_evaluations_per_s": round(chains * dsteps / dwall, 1)},
            "launch": "one CUDA graph per step: staged copies, one transition kernel, one "
                      "persistent pruning kernel, read-back"}


def protein20(device: int, steps: int, warmup: int, seed: int = 4, L: int = 128,
              N: int = 5000, forms=("f32", "f64")) -> dict:
    """The 20-state workload: 128 taxa, 5,000 sites, exchangeabilities
    r_ij ~ LogNormal(0, 1) (190 values), pi ~ Dir(1 x 20), Gamma4 alpha = 1,
    simulated down a seeded Yule tree.  Whole-tree evaluations of both
    forms, device time per evaluation from CUDA events; GB/s counts the
    algorithmic bytes with S = 20, TFLOP/s the algorithmic flops
    sum_v C P (2 S^2 per internal child + S)."""
    from aspartik_gb300.calculator import Calculator

    rng = np.random.default_rng(seed)
    K = 4
    tree = sim.yule_tree(L, rng, root_height=1.0)
    pi = sim.dirichlet([1.0] * 20, rng)
    pi = np.maximum(pi, 1e-4)
    pi /= pi.sum()
    rates = rng.lognormal(0.0, 1.0, size=190)
    Q = sim.reversible_q(rates, pi)
    states = sim.simulate_alignment(tree, N, Q, pi, rng, cat_rates=sim.gamma_rates(1.0, K))
    leaves, weights, _ = sim.deduplicate(states, dna=False)
    P = leaves.shape[1]
    top = schedule.Topology(tree.parents, tree.heights)
    lists = top.full()
    ch = top.children[np.asarray(lists[0], dtype=np.int64) - top.L]
    n_int = int((ch >= top.L).sum())
    flops = K * P * (n_int * 2 * 20 * 20 + len(lists[0]) * 20)
    out = {"workload": f"prot{L}x{N}_rev20_g4", "taxa": L, "sites": N, "patterns": P,
           "categories": K, "states": 20}
    for form in forms:
        precision = "f64" if form == "f64" else "f32"
        w = 8 if precision == "f64" else 4
        old_env = os.environ.get("B3G_TC20")
        if form == "f32_cuda_cores":
            os.environ["B3G_TC20"] = "0"
        try:
            calc = Calculator.GB300(device, precision).make20(leaves, P, num_categories=K)
        finally:
            if old_env is None:
                os.environ.pop("B3G_TC20", None)
            else:
                os.environ["B3G_TC20"] = old_env
        calc.set_weights(weights)
        calc.set_reversible(rates, pi)
        calc.set_gamma(1.0)
        engine = "CUDA cores" if form == "f32_cuda_cores" else None
        if form == "f32":
            calc.propose_lengths(*lists, 1.0)
            calc.log_likelihood()
            calc.accept()
            engine = "tensor cores" if calc.autotune(*lists, 1.0) else "CUDA cores"
        k = steps if precision == "f32" else max(3, min(steps, 20))
        ms, _, prune_ms, _ = device_throughput(calc, lists, k, warmup, 1)
        lnl = calc.log_likelihood()
        calc.close()
        b = schedule.algorithmic_bytes(top, lists[0], P, K, 20, w=w, e_b=4, w_p=w)
        out[form] = {"ms_per_eval": round(ms / k, 5), "kernel_ms": round(prune_ms, 5),
                          "bytes_per_eval": b, "GB_s": round(b / (ms / k * 1e-3) / 1e9, 2),
                          "kernel_GB_s": round(b / (prune_ms * 1e-3) / 1e9, 2),
                          "kernel_TFLOP_s": round(flops / (prune_ms * 1e-3) / 1e12, 3),
                          "lnl": lnl}
        if engine:
            out[form]["engine"] = engine
    out["flops_per_eval"] = flops
    if "f64" in out:
        out["lnl_rel_err_f32_vs_f64"] = abs(out["f32"]["lnl"] - out["f64"]["lnl"]) / abs(
            out["f64"]["lnl"])
    if "f32_cuda_cores" in out:
        out["lnl_rel_diff_tensor_vs_cuda_cores"] = abs(
            out["f32"]["lnl"] - out["f32_cuda_cores"]["lnl"]) / abs(out["f32_cuda_cores"]["lnl"])
    return out


ESS_FIELDS = ("lnl", "root_height", "kappa_or_rate0")


def mcmc_settings(wl, precision: str, **kw):
    from aspartik_gb300.mcmc import GTR_WEIGHTS, HKY_SCALE_KAPPA_WEIGHTS, McmcSettings

    spec = wl["spec"]
    weights = GTR_WEIGHTS if spec["model"] == "gtr" else HKY_SCALE_KAPPA_WEIGHTS
    kw.setdefault("weights", dict(weights))
    return McmcSettings(model=spec["model"], precision=precision,
                        num_categories=spec["categories"], sample_every=10, **kw)


def start_parameters(wl) -> dict:
    """The simulated tree and parameters."""
    return dict(parents=wl["tree"].parents, heights=wl["tree"].heights,
                rates=wl["rates"] if wl["spec"]["model"] == "gtr" else None, freqs=wl["pi"],
                kappa=2.0, alpha=wl["spec"]["alpha"] or 1.0, birth=1.0)


def burn_in(wl, steps: int, device: int) -> tuple[dict, dict, float]:
    """A chosen-form chain from the simulated tree and parameters; its final
    state and operator tunings start every measured arm, so that each arm
    samples near stationarity from its first step."""
    from aspartik_gb300.mcmc import Mcmc

    st = start_parameters(wl)
    m = Mcmc(wl["leaves"], wl["weights"], st["parents"], st["heights"],
             mcmc_settings(wl, "f32", seed=3, device=device))
    m.set_parameters(kappa=st["kappa"], rates=st["rates"], frequencies=st["freqs"],
                     alpha=st["alpha"], birth_rate=st["birth"])
    t0 = time.perf_counter()
    m.run(steps)
    dt = time.perf_counter() - t0
    smp = m.samples()
    tunings = {k: v["tuning"] for k, v in m.operator_stats().items()}
    m.close()
    start = dict(parents=smp["parents"][-1], heights=smp["heights"][-1],
                 rates=smp["rates"][-1] if wl["spec"]["model"] == "gtr" else None,
                 freqs=smp["frequencies"][-1], kappa=float(smp["kappa"][-1]),
                 alpha=float(smp["alpha"][-1]), birth=float(smp["birth_rate"][-1]))
    return start, tunings, dt


def mcmc_arm(wl, start, tunings, precision: str, steps: int, device: int, chains: int = 1,
             da_pilot: int = 0, burn_frac: float = 0.05, seed: int = 4,
             launch: str = "streams") -> dict:
    """One arm of the ESS/s comparison: `chains` chains (independent
    replicates stepping together) from `start`, `steps` steps, wall time of
    the whole run (pilot and surrogate training included).  ESS of lnL, root
    height and the first exchangeability (kappa for HKY) by Geyer's initial
    monotone sequence (one chain) or the multi-chain estimator of BDA3 11.5
    (replicates: their disagreement counts against them), after dropping the
    first `burn_frac` of the samples."""
    from aspartik_gb300.ess import min_ess, multi_chain_ess
    from aspartik_gb300.mcmc import Mcmc

    kw = dict(seed=seed, device=device, num_chains=chains, heat=0.0, swap_every=0,
              launch=launch)
    if da_pilot:
        kw.update(da_pilot_steps=da_pilot, da_epochs=100, da_hidden=256, da_drift_limit=20.0)
    m = Mcmc(wl["leaves"], wl["weights"], start["parents"], start["heights"],
             mcmc_settings(wl, precision, **kw))
    m.set_parameters(kappa=start["kappa"], rates=start["rates"], frequencies=start["freqs"],
                     alpha=start["alpha"], birth_rate=start["birth"])
    if tunings:
        m.set_tuning(tunings)
    t0 = time.perf_counter()
    m.run(steps)
    dt = time.perf_counter() - t0
    n = m.trace("lnl").size
    keep = int(n * burn_frac)
    if chains == 1:
        traces = {k: m.trace(k)[keep:] for k in ESS_FIELDS}
        e, per = min_ess(traces, burn_in=0.0)
    else:
        per = {k: multi_chain_ess([m.trace(k, chain=c)[keep:] for c in range(chains)],
                                  burn_in=0.0) for k in ESS_FIELDS}
        e = min(per.values())
        traces = {"lnl": np.concatenate([m.trace("lnl", chain=c)[keep:]
                                         for c in range(chains)])}
    out = {"chains": chains, "launch": launch, "steps": steps, "seconds": round(dt, 3),
           "us_per_step": round(dt / steps * 1e6, 2),
           "chain_steps_per_s": round(chains * steps / dt, 1),
           "ess_min": round(e, 1), "ess": {k: round(v, 1) for k, v in per.items()},
           "ess_per_s": round(e / dt, 3), "mean_lnl": float(np.mean(traces["lnl"])),
           "check_rel": m.check()}
    if da_pilot:
        out["delayed_acceptance"] = m.da_stats()
    m.close()
    return out


def mcmc_ess(wl, chosen_steps: int, device: int) -> dict:
    """ESS per second, chosen form against the plain FP64 form, on the
    workload, every arm started from the same burned-in state and operator
    tunings (a chosen-form chain of chosen_steps / 7.5 steps from the
    simulated tree and parameters, not timed in any arm):
      plain_f64                one chain, FP64 partials (the drop-in's
                               arithmetic), 0.4 x chosen_steps steps
      chosen_f32               one chain, FP32 power-of-two-scaled partials
      chosen_f32_da            one chain with delayed acceptance: the first
                               10^5 steps are the pilot, then the surrogate
                               (trained on the GPU) screens the moves that
                               re-evaluate the whole tree
      chosen_f32_da_replicates the chosen form in full: 8 independent
                               replicates, each on its own host thread and
                               stream, advancing on their own between the
                               driver's synchronisation points (operator
                               tuning, the pilot's end), with delayed
                               acceptance (pilot: the first 1/16 of the
                               steps), chosen_steps / 3.75 steps (each
                               chain long enough that the multi-chain ESS,
                               which counts the chains' disagreement, is
                               not dominated by it), multi-chain ESS
    Moves: the driver's GTR mix (tree scale 3, subtree slide 30, narrow
    exchange 30, wide exchange 3, root slide 3, node slide 30, up-down 3,
    alpha scale 1, birth-rate scale 3, delta exchange of rates 1 and of
    frequencies 1)."""
    burn = int(chosen_steps / 7.5)
    start, tunings, burn_s = burn_in(wl, burn, device)
    out = {"burn_in": {"steps": burn, "seconds": round(burn_s, 3), "form": "f32",
                       "tunings": {k: round(v, 6) for k, v in tunings.items()}}}
    progress("MCMC burn-in")
    out["plain_f64"] = mcmc_arm(wl, start, tunings, "f64", int(0.4 * chosen_steps), device)
    progress("MCMC plain FP64 arm")
    out["chosen_f32"] = mcmc_arm(wl, start, tunings, "f32", chosen_steps, device)
    progress("MCMC chosen FP32 arm")
    out["chosen_f32_da"] = mcmc_arm(wl, start, tunings, "f32", chosen_steps, device,
                                    da_pilot=min(100_000, chosen_steps // 5))
    progress("MCMC delayed-acceptance arm")
    rep = int(chosen_steps / 3.75)
    out["chosen_f32_da_replicates"] = mcmc_arm(wl, start, tunings, "f32", rep, device,
                                               chains=8, da_pilot=rep // 16,
                                               launch="independent")
    progress("MCMC replicates arm")
    base = max(out["plain_f64"]["ess_per_s"], 1e-12)
    for arm in ("chosen_f32", "chosen_f32_da", "chosen_f32_da_replicates"):
        out[f"ess_per_s_ratio_{arm}_vs_plain"] = round(out[arm]["ess_per_s"] / base, 3)
    out["ess_min_all_arms"] = min(out[a]["ess_min"] for a in
                                  ("plain_f64", "chosen_f32", "chosen_f32_da",
                                   "chosen_f32_da_replicates"))
    out["mean_lnl_rel_diff_chosen_vs_plain"] = abs(
        out["chosen_f32"]["mean_lnl"] - out["plain_f64"]["mean_lnl"]) / abs(
        out["plain_f64"]["mean_lnl"])
    out["ess_fields"] = list(ESS_FIELDS)
    return out


def config_block(name: str, device: int, mcmc_steps: int, reps: int = 50) -> dict:
    """One of the smaller configurations on its own: whole-tree evaluation
    time of both forms (device time, CUDA events), the log-likelihood of
    each against the restated cpu4 (oracle/b3oracle.c, the CPU baseline of
    this block, timed on all host threads), and the ESS/s of the chosen form
    against the plain FP64 form over `mcmc_steps` steps from the simulated
    tree (10% burn-in dropped)."""
    wl = make_workload(name)
    spec = wl["spec"]
    top = wl["top"]
    P = int(wl["leaves"].shape[1])
    C = spec["categories"]
    full = top.full()
    out = {"taxa": spec["taxa"], "sites": spec["sites"], "patterns": P, "categories": C,
           "model": spec["model"]}
    lnl = {}
    for precision, w in (("f32", 4), ("f64", 8)):
        calc = make_calc(wl, precision, device)
        if precision == "f32":
            calc.propose_lengths(*full, 1.0)
            calc.log_likelihood()
            calc.accept()
            calc.autotune(*full, 1.0)
        ms, _, prune_ms, _ = device_throughput(calc, full, reps, 5, 1)
        lnl[precision] = calc.log_likelihood()
        calc.close()
        B = schedule.algorithmic_bytes(top, full[0], P, C, 4, w=w, e_b=4, w_p=w)
        out[f"whole_tree_{precision}"] = {
            "ms_per_eval": round(ms / reps, 5), "kernel_ms": round(prune_ms, 5),
            "GB_s": round(B / (ms / reps * 1e-3) / 1e9, 2), "bytes_per_eval": B,
            "lnl": lnl[precision]}
    cores = os.cpu_count() or 1
    ref = CpuReference(wl, cores)
    ref.evaluate()
    t_cpu, cpu_lnl = ref.evaluate()
    out["cpu_baseline"] = {"kind": "port", "cores": ref.threads,
                           "ms_per_eval": round(t_cpu * 1e3, 3), "lnl": cpu_lnl,
                           "sample": "one whole-tree evaluation of the full alignment; "
                                     "cpu4-restated, FP64, e^30 rescaling"}
    out["lnl_rel_err_f64_vs_oracle"] = abs(lnl["f64"] - cpu_lnl) / abs(cpu_lnl)
    out["lnl_rel_err_f32_vs_oracle"] = abs(lnl["f32"] - cpu_lnl) / abs(cpu_lnl)
    if mcmc_steps > 0:
        st = start_parameters(wl)
        arms = {p: mcmc_arm(wl, st, None, p, mcmc_steps, device, burn_frac=0.1)
                for p in ("f64", "f32")}
        out["mcmc"] = {"steps": mcmc_steps, "plain_f64": arms["f64"], "chosen_f32": arms["f32"],
                       "ess_per_s_ratio_chosen_vs_plain": round(
                           arms["f32"]["ess_per_s"] / max(arms["f64"]["ess_per_s"], 1e-12), 3),
                       "moves": "tree scale 3, kappa scale 1" if spec["model"] == "hky" else
                       "the GTR mix of the MCMC leg (NNI = narrow exchange, subtree slide)"}
    return out


def c4_problems(seed: int = 4, problems: int = 4) -> list:
    """The batched configuration's alignments: taxa uniform on 24..200, sites
    log-uniform on 500..50,000, each simulated under GTR + Gamma4 as the
    64-taxon configuration (exchangeabilities ~ Gamma(2, 1), frequencies ~
    Dirichlet(5, 5, 5, 5), alpha 0.5) down a Yule tree of root height 1."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(problems):
        L = int(rng.integers(24, 201))
        N = int(np.exp(rng.uniform(np.log(500), np.log(50000))))
        tree = sim.yule_tree(L, rng, root_height=1.0)
        pi = sim.dirichlet([5.0] * 4, rng)
        rates = rng.gamma(2.0, 1.0, size=6)
        states = sim.simulate_alignment(tree, N, sim.reversible_q(rates, pi), pi, rng,
                                        cat_rates=sim.gamma_rates(0.5, 4))
        leaves, weights, _ = sim.deduplicate(sim.to_dna_codes(states))
        out.append(dict(taxa=L, sites=N, patterns=int(leaves.shape[1]), leaves=leaves,
                        weights=weights, tree=tree))
    return out


def c4_mcmc(device: int, steps: int, temps: int = 8) -> dict:
    """The batched configuration as an MCMC: 4 alignments (c4_problems) x 8
    MC3 temperatures, beta_i = 1 / (1 + 0.1 i), = 32 FP32 chains of uneven
    taxa and sites in one driver (b3g_mcmc_create_multi), swap attempts
    every 10 steps within each alignment's ladder, the GTR moves of the MCMC
    leg.  Run once per launch mode: every chain's evaluations of a step in
    one graph replay of the batched kernels (one staging copy, the run walk
    for long lists, the batched short-list kernel, one read-back), or one
    launch per chain on its own stream, the chains spread over host threads
    (one for every four chains, at most 8), or the same with each thread
    advancing its chains on their own between swap attempts (independent
    stepping, 8 threads).  Wall time per step and, batched,
    the graph's device time per step (CUDA events); ESS of the cold chain of
    the first alignment (lnL, root height, first exchangeability)."""
    from aspartik_gb300.ess import min_ess
    from aspartik_gb300.mcmc import GTR_WEIGHTS, Mcmc, McmcSettings

    probs = c4_problems()
    out = {"problems": [{k: p[k] for k in ("taxa", "sites", "patterns")} for p in probs],
           "chains": temps * len(probs), "temperatures": temps, "steps": steps,
           "host_threads_streams": min((temps * len(probs) + 3) // 4, 8, os.cpu_count() or 1)}
    for launch in ("batch", "streams", "independent"):
        s = McmcSettings(model="gtr", precision="f32", num_categories=4,
                         num_chains=temps * len(probs), heat=0.1, swap_every=10, seed=4,
                         sample_every=10, weights=dict(GTR_WEIGHTS), device=device,
                         launch=launch)
        m = Mcmc.multi([(p["leaves"], p["weights"], p["tree"].parents, p["tree"].heights)
                        for p in probs], s)
        m.set_parameters(rates=np.ones(6), frequencies=np.full(4, 0.25), alpha=0.5,
                         birth_rate=1.0)
        m.run(200)  # warm-up: operator tuning, first graph replays
        st0 = m.launch_stats()
        tried0, acc0 = m.swaps()
        t0 = time.perf_counter()
        m.run(steps)
        dt = time.perf_counter() - t0
        st = m.launch_stats()
        tried, acc = m.swaps()
        keep = (steps // 10) // 5
        traces = {k: m.trace(k)[20 + keep:] for k in ESS_FIELDS}
        e, per = min_ess(traces, burn_in=0.0)
        arm = {"seconds": round(dt, 3), "wall_us_per_step": round(dt / steps * 1e6, 2),
               "chain_steps_per_s": round(temps * len(probs) * steps / dt, 1),
               "swap_rate": round((acc - acc0) / max(tried - tried0, 1), 3),
               "cold_chain_ess_min": round(e, 2),
               "cold_chain_ess": {k: round(v, 2) for k, v in per.items()},
               "check_rel": m.check()}
        if st["batched"]:
            n = st["launches"] - st0["launches"]
            dev_us = (st["device_ms"] - st0["device_ms"]) * 1e3 / max(n, 1)
            arm["graph_replays"] = n
            arm["device_us_per_step"] = round(dev_us, 2)
            arm["wall_over_device"] = round(arm["wall_us_per_step"] / max(dev_us, 1e-9), 3)
        out[launch] = arm
        m.close()
    out["faster"] = min(("batch", "streams", "independent"),
                        key=lambda k: out[k]["wall_us_per_step"])
    return out


def dedup_leg(device: int, seed: int = 4) -> dict:
    """Site-pattern compression of the largest batched configuration's
    alignment size (200 taxa x 50,000 sites, simulated under GTR) on the
    GPU; CPU baseline: the restated deduplicate (hash map, one thread)."""
    from aspartik_gb300.calculator import deduplicate
    from oracle import oracle as O

    rng = np.random.default_rng(seed)
    tree = sim.yule_tree(200, rng, root_height=0.5)
    pi = sim.dirichlet([5.0] * 4, rng)
    Q = sim.reversible_q(rng.gamma(2.0, 1.0, 6), pi)
    msa = sim.to_dna_codes(sim.simulate_alignment(tree, 50000, Q, pi, rng))
    deduplicate(msa, device=device)  # warm-up
    dev, wall = [], []
    for _ in range(5):
        t0 = time.perf_counter()
        leaves, weights, s2p, ms = deduplicate(msa, device=device)
        wall.append(time.perf_counter() - t0)
        dev.append(ms)
    t0 = time.perf_counter()
    ol, ow, os_ = O.deduplicate(msa)
    t_cpu = time.perf_counter() - t0
    same = bool(np.array_equal(leaves, ol) and np.array_equal(weights, ow)
                and np.array_equal(s2p, os_))
    return {"taxa": 200, "sites": 50000, "patterns": int(weights.size),
            "device_ms": round(statistics.median(dev), 4),
            "e2e_ms": round(statistics.median(wall) * 1e3, 4),
            "alignment_GB_s": round(msa.nbytes / (statistics.median(dev) * 1e-3) / 1e9, 2),
            "cpu_baseline_ms": round(t_cpu * 1e3, 3), "identical_to_cpu": same}


def mc3(wl, steps: int, device: int, chains: int = 8, launch: str = "independent") -> dict:
    """Metropolis-coupled MCMC on the workload: `chains` FP32 chains at
    beta_i = 1 / (1 + 0.1 i), swap attempts every 10 steps, the moves of
    mcmc_ess.  Every chain launches its own evaluations on its own stream;
    with independent stepping (the default here) each host thread advances
    its chains on their own between swap attempts, otherwise all chains'
    evaluations of a step are queued before any result is read."""
    from aspartik_gb300.ess import min_ess
    from aspartik_gb300.mcmc import Mcmc

    s = mcmc_settings(wl, "f32", num_chains=chains, heat=0.1, swap_every=10, seed=4,
                      device=device, launch=launch)
    m = Mcmc(wl["leaves"], wl["weights"], wl["tree"].parents, wl["tree"].heights, s)
    m.set_parameters(rates=wl["rates"], frequencies=wl["pi"],
                     alpha=wl["spec"]["alpha"] or 1.0, birth_rate=1.0)
    m.run(min(200, steps))  # warm-up (operator tuning)
    t0 = time.perf_counter()
    m.run(steps)
    dt = time.perf_counter() - t0
    tried, accepted = m.swaps()
    keep = (steps // 10) // 5
    traces = {k: m.trace(k)[keep:] for k in ESS_FIELDS}
    e, _ = min_ess(traces, burn_in=0.0)
    out = {"chains": chains, "launch": launch, "steps": steps, "seconds": round(dt, 3),
           "us_per_step": round(dt / steps * 1e6, 2),
           "chain_steps_per_s": round(chains * steps / dt, 1),
           "swaps_tried": tried, "swaps_accepted": accepted,
           "cold_chain_ess_min": round(e, 2), "check_rel": m.check()}
    m.close()
    return out


def run_ours(args):
    world, rank, local = dist_setup()
    device = local
    wl = make_workload(args.workload)
    spec = wl["spec"]
    top = wl["top"]
    P = int(wl["leaves"].shape[1])
    C = spec["categories"]
    full = top.full()
    I = top.L - 1
    B32 = schedule.algorithmic_bytes(top, full[0], P, C, 4, w=4, e_b=4, w_p=4)
    B64 = schedule.algorithmic_bytes(top, full[0], P, C, 4, w=8, e_b=4, w_p=8)
    pk = peaks()

    calc = make_calc(wl, "f32", device)
    # the library's autotuner picks the tile size of the whole-tree walk
    # (trial evaluations are rejected; outside the timed region)
    calc.propose_lengths(*full, 1.0)
    calc.log_likelihood()
    calc.accept()
    tile = calc.autotune(*full, 1.0)
    clocks = ClockSampler(device)
    clocks.start()
    time.sleep(0.3)
    ms, t_tr, t_pr, nlaunch = device_throughput(calc, full, args.steps, args.warmup, world)
    kernels_per_eval = calc.last_launches()
    clk = clocks.stop()
    progress("whole-tree throughput")
    ms_max = allreduce_max(ms, world)
    value = world * args.steps * B32 / (ms_max * 1e-3) / 1e9
    achieved = B32 / (t_pr * 1e-3) / 1e9

    # e2e: host buffers in, log-likelihood out, blocking every step
    internals, children, lengths = full
    barrier(world)
    t0 = time.perf_counter()
    lnl = None
    for _ in range(args.steps):
        calc.propose_lengths(internals, children, lengths, 1.0)
        lnl = calc.log_likelihood()
    e2e_s = allreduce_max(time.perf_counter() - t0, world)
    h2d = calc.last_upload_bytes()
    e2e = world * args.steps * B32 / e2e_s / 1e9

    # dirty path: height change of a random internal node
    rng = np.random.default_rng(7)
    nodes = rng.integers(top.L, 2 * top.L - 1, size=min(args.steps, 512))
    paths = [top.path(int(v)) for v in nodes]
    for p in paths[:args.warmup]:
        calc.propose_lengths(*p, 1.0)
    calc.log_likelihood()
    calc.span_begin()
    for p in paths:
        calc.propose_lengths(*p, 1.0)
    dms = calc.span_end()
    calc.set_timing(True)
    calc.timing_totals(reset=True)
    for p in paths:
        calc.propose_lengths(*p, 1.0)
    calc.log_likelihood()
    _, dprune, dn = calc.timing_totals(reset=True)
    calc.set_timing(False)
    dbytes = sum(schedule.algorithmic_bytes(top, p[0], P, C, 4, w=4, e_b=4, w_p=4) for p in paths)
    mean_path = float(np.mean([len(p[0]) for p in paths]))
    calc.close()
    progress("e2e and dirty path")

    # plain FP64 form, same workload
    c64 = make_calc(wl, "f64", device)
    k64 = max(3, min(args.steps, 200))
    ms64, _, pr64, _ = device_throughput(c64, full, k64, args.warmup, world)
    lnl64 = c64.log_likelihood()
    c64.close()
    progress("plain FP64 whole tree")

    # the MCMC legs run once, on the single-GPU run (replicas add nothing)
    long_legs = world == 1 and args.mcmc_steps > 0
    mcmc = mcmc_ess(wl, args.mcmc_steps, device) if long_legs else None
    mc3_out = mc3(wl, 5000, device) if long_legs else None
    if long_legs:
        progress("MC3")
    c4 = c4_mcmc(device, 20_000) if long_legs else None
    if long_legs:
        progress("32-chain MCMC (4 alignments x 8 temperatures)")
    configs = None
    if long_legs and args.workload == DEFAULT_WORKLOAD:
        configs = {"dna16x1000_hky": config_block("dna16x1000_hky", device, 10_000)}
        progress("16-taxon configuration")
        configs["dna64x10000_gtr_g4"] = config_block("dna64x10000_gtr_g4", device, 100_000)
        progress("64-taxon configuration")
    dedup = None if args.no_cpu else dedup_leg(device)
    progress("deduplication")
    prot = prot_big = None
    if not args.no_protein:
        prot = protein20(device, min(args.steps, 100), args.warmup)
        prot_big = protein20(device, min(args.steps, 20), args.warmup, N=50000,
                             forms=("f32", "f32_cuda_cores"))
    progress("20 states")
    batch = None if args.no_batch else batched(device, min(args.steps, 200), args.warmup)
    progress("batched chains")

    cpu = None
    if rank == 0 and not args.no_cpu:
        cores = os.cpu_count() or 1
        ref = CpuReference(wl, cores)
        dt1, cpu_lnl = ref.evaluate()
        reps = int(max(1, min(20, 5.0 / max(dt1, 1e-3))))
        times = [ref.evaluate()[0] for _ in range(reps)]
        t_cpu = statistics.median(times)
        Pu, thr = ref.P, ref.threads
        # the reference's own default thread count (cpu4.rs:126-131)
        default_thr = min(cores, -(-Pu // 1000))
        t_def = t_cpu
        if default_thr != thr:
            ref_def = CpuReference(wl, default_thr)
            t_def = statistics.median([ref_def.evaluate()[0] for _ in range(reps)])
        cpu = {"value": round(B32 / t_cpu / 1e9, 4), "unit": UNIT, "cores": thr,
               "kind": "port",
               "sample": f"{reps} whole-tree evaluations of the full workload ({Pu} patterns x "
                         f"{C} categories), median {t_cpu * 1e3:.1f} ms each; cpu4-restated "
                         f"(reference Rust not buildable): FP64, e^30 rescaling, one calculator "
                         f"per category, {thr} threads",
               "ms_per_eval": round(t_cpu * 1e3, 3),
               "default_threads": default_thr,
               "value_default_threads": round(B32 / t_def / 1e9, 4),
               "lnl_rel_err_vs_gpu_f64": abs(cpu_lnl - lnl64) / abs(cpu_lnl)}

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_max / args.steps, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Yule tree + GTR+Gamma4 simulated alignment, seed 4)",
        "config": {"workload": args.workload, "taxa": spec["taxa"], "sites": spec["sites"],
                   "patterns": P, "categories": C, "states": 4,
                   "evaluation": "whole tree (all internals dirty)",
                   "bytes_per_step": B32,
                   "l2": "inputs larger than L2 (FP32 partials %.2f GB)"
                         % (2 * I * C * P * 16 / 1e9),
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4),
                     "traffic": TRAFFIC_RUNS_BYTES if args.workload == DEFAULT_WORKLOAD else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                       "one whole-tree launch of this workload",
                     "peak_source": pk["source"],
                     "kernel": "prune4_runs_kernel (FP32, run-synchronous)",
                     "tile_patterns": tile,
                     "kernel_ms": round(t_pr, 5), "transition_kernel_ms": round(t_tr, 5)},
        "e2e": {"value": round(e2e, 2), "unit": UNIT,
                "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 8, "ms_per_step": round(e2e_s * 1e3 / args.steps, 5)},
        "gpu_launches": int(nlaunch * kernels_per_eval),
        "clocks": clk,
        "lnl": lnl,
        "plain_f64": {"value": round(k64 * B64 / (ms64 * 1e-3) / 1e9, 2),
                      "ms_per_step": round(ms64 / k64, 5),
                      "kernel_ms": round(pr64, 5), "bytes_per_step": B64,
                      "lnl": lnl64, "f32_rel_err": abs(lnl - lnl64) / abs(lnl64)},
        "dirty_path": {"value": round(dbytes / (dms * 1e-3) / 1e9, 2),
                       "us_per_eval": round(dms * 1e3 / len(paths), 3),
                       "mean_nodes": mean_path,
                       "kernel_us": round(dprune * 1e3 / max(dn, 1), 3)},
        "mcmc": mcmc,
        "mc3": mc3_out,
        "c4_mcmc": c4,
        "configs": configs,
        "dedup": dedup,
        "batched": batch,
        "protein20": prot,
        "protein20_large": prot_big,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))


def reference_cuda(wl, workload: str, reps: int = 20) -> dict:
    """The reference's own FP64 CUDA calculators on the same GPU: the
    kernels of crates/b3/src/calculator/cuda_partials and cuda_propagations
    (its default GPU calculator), compiled unchanged from the reference tree
    into oracle/_ref by oracle/build.py::build_ref and driven as the
    reference's calculators drive them (oracle/ref_cuda.py).  One
    evaluation of the reference's GammaLikelihood is one whole-tree
    calculator evaluation per Gamma category (likelihood/gamma.rs:97-169);
    device time of the launches with the inputs resident, and GB/s by the
    FP64 byte formula with one-byte scale flags."""
    try:
        from oracle import oracle as O
        from oracle import ref_cuda
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"reference CUDA driver not importable: {e}"}
    if not (ref_cuda.available() and ref_cuda.propagations_available()):
        return {"unavailable": "reference CUDA kernels not built (oracle/_ref)"}
    spec = wl["spec"]
    C = spec["categories"]
    model = O.gtr(wl["rates"], wl["pi"])
    cats = O.gamma_categories(spec["alpha"], C) if spec["alpha"] else np.ones(1)
    internals, children, lengths = wl["top"].full()
    P = int(wl["leaves"].shape[1])
    L = int(wl["leaves"].shape[0])
    per_cat, per_cat_prop = [], []
    part = ref_cuda.RefCudaPartials(0)
    try:
        part.setup(ref_cuda.dna_codes_to_ref(wl["leaves"]), 30)
        for r in cats:
            mats = np.array([[model.transition(d * r) for d in pair] for pair in lengths])
            part.propose(internals, children, mats, wl["pi"])
            part.result()
            part.time_last(3)  # warm-up
            per_cat.append(part.time_last(reps))
    finally:
        part.close()
    prop = ref_cuda.RefCudaPropagations(0)
    try:
        prop.setup(wl["leaves"], 30)
        for r in cats:
            nodes, k, pch, pmats = ref_cuda.propagation_inputs(wl["tree"], model, r, L)
            prop.propose(nodes, k, pch, pmats, wl["pi"])
            prop.result()
            prop.time_last(3)
            per_cat_prop.append(prop.time_last(reps))
    finally:
        prop.close()
    ms, ms_prop = float(sum(per_cat)), float(sum(per_cat_prop))
    B64 = schedule.algorithmic_bytes(wl["top"], internals, P, C, 4, w=8, e_b=1, w_p=8)
    return {"workload": workload, "patterns": P, "categories": C,
            "partials": {"kernel_ms_per_category": [round(x, 4) for x in per_cat],
                         "ms_per_evaluation": round(ms, 4),
                         "GB_s": round(B64 / (ms * 1e-3) / 1e9, 2)},
            "propagations": {"kernel_ms_per_category": [round(x, 4) for x in per_cat_prop],
                             "ms_per_evaluation": round(ms_prop, 4),
                             "GB_s": round(B64 / (ms_prop * 1e-3) / 1e9, 2)},
            "note": "reference CUDA calculators, FP64: partials (one launch per category, one "
                    "thread per pattern) and propagations, the default (leaf, propagation "
                    "and root kernels per category, four threads per pattern); device time, "
                    "inputs resident, whole tree; GB/s by the FP64 byte formula"}


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    wl = make_workload(args.workload)
    spec = wl["spec"]
    top = wl["top"]
    P = int(wl["leaves"].shape[1])
    C = spec["categories"]
    full = top.full()
    cores = os.cpu_count() or 1
    # bound the run: each step's pattern sample is sized so that warmup +
    # steps take about a minute of evaluation at most
    dt1, _ = CpuReference(wl, cores).evaluate()
    budget = 60.0
    frac = min(1.0, budget / max(dt1 * (args.steps + args.warmup), 1e-9))
    Pu = max(128, int(P * frac)) if frac < 1.0 else P
    ref = CpuReference(wl, cores, Pu)
    thr = ref.threads
    for _ in range(args.warmup):
        ref.evaluate()
    total = 0.0
    for _ in range(args.steps):
        total += ref.evaluate()[0]
    B = schedule.algorithmic_bytes(top, full[0], Pu, C, 4, w=4, e_b=4, w_p=4)
    value = args.steps * B / total / 1e9
    sample = (f"whole-tree evaluations over {Pu} of {P} patterns x {C} categories per step; "
              f"cpu4-restated (reference Rust not buildable): FP64, e^30 rescaling, "
              f"{thr} threads")
    # beside it, the reference's own CUDA calculators on this GPU
    ref_gpu = {"unavailable": "no CUDA device"}
    try:
        import torch

        if torch.cuda.is_available():
            ref_gpu = reference_cuda(wl, args.workload)
    except Exception as e:  # noqa: BLE001
        ref_gpu = {"unavailable": f"{type(e).__name__}: {e}"}
    print(json.dumps({
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total * 1e3 / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": "synthetic (seeded Yule tree + GTR+Gamma4 simulated alignment, seed 4)",
        "config": {"workload": args.workload, "taxa": spec["taxa"], "sites": spec["sites"],
                   "patterns": P, "categories": C, "sampled_patterns": Pu,
                   "bytes_per_step": B,
                   "note": "reference Rust workspace not buildable here; its CPU pruner "
                           "restated in C (oracle/b3oracle.c)"},
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": thr, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "reference_cuda": ref_gpu,
    }))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-chains leg")
    ap.add_argument("--no-protein", action="store_true", help="skip the 20-state leg")
    ap.add_argument("--mcmc-steps", type=int, default=1_500_000,
                    help="steps of the chosen-form MCMC arms of the ESS/s comparison; the "
                         "plain arm runs 0.4x, burn-in 1/7.5x and replicates 1/3.75x (0 = skip the "
                         "MCMC legs and the smaller configurations)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
