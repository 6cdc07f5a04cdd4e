"""Python face of the native MCMC driver (``b3g_mcmc_*`` in include/b3g.h).

The driver restates the step of b3's engine (crates/b3/src/mcmc.rs:314-393)
in C++ around the device likelihood; this wrapper only configures it, runs
it and reads its traces.
"""

from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass, field

import numpy as np

from . import _native as nat
from ._native import check, lib

MODELS = {"hky": 0, "gtr": 1}
OPERATORS = ["tree_scale", "subtree_slide", "narrow_exchange", "scale_kappa",
             "scale_alpha", "scale_birth_rate", "delta_rates", "delta_frequencies",
             "relaxed_category", "scale_clock_sd", "node_slide", "root_slide", "up_down",
             "wide_exchange"]
# parameters of a state file in the reference's layout (B3G_STATE_*)
STATE_PARAMETERS = ["tree", "birth_rate", "kappa", "alpha", "rates", "frequencies",
                    "clock_sd", "clock_categories"]
TRACE_FIELDS = ["lnl", "prior", "posterior", "root_height", "kappa_or_rate0", "alpha",
                "tree_length", "clock_sd"]

# the operator mix of the reference's config recipe for a Yule + GTR model:
# the tree operators of its "beauti1_classic" mix (TreeScale 3, SubtreeSlide
# 30, BeastNarrowExchange 30, BeastWideExchange 3, RootSlide 3, NodeSlide 30;
# python/aspartik/b3/config/__init__.py:849-858), UpDown of the tree against
# the Yule birth rate (the pairing of the "beauti1_default" mix, :835-845,
# with the birth rate in place of the clock rate) and the parameter
# operators of the recipe (:660-730)
GTR_WEIGHTS = dict(tree_scale=3, subtree_slide=30, narrow_exchange=30, wide_exchange=3,
                   root_slide=3, node_slide=30, up_down=3, scale_alpha=1, scale_birth_rate=3,
                   delta_rates=1, delta_frequencies=1)
# branch-length scale and kappa moves only
HKY_SCALE_KAPPA_WEIGHTS = dict(tree_scale=3, scale_kappa=1)


@dataclass
class McmcSettings:
    model: str = "gtr"
    precision: str = "f32"
    num_categories: int = 4
    num_chains: int = 1
    seed: int = 4
    heat: float = 0.0
    swap_every: int = 0
    sample_every: int = 10
    tune_every: int = 1000
    device: int = 0
    weights: dict = field(default_factory=lambda: dict(GTR_WEIGHTS))
    # delayed acceptance (0 pilot steps: off)
    da_pilot_steps: int = 0
    da_epochs: int = 20
    da_hidden: int = 256
    da_drift_limit: float = 0.0
    # relaxed clock: rate categories per edge (0: strict clock)
    clock_categories: int = 0
    # "streams": one launch per chain on its own stream; "batch": every
    # chain of a step in one graph-replayed batched launch (FP32);
    # "independent": streams, chains advancing on their own between swap
    # attempts and tuning points
    launch: str = "streams"
    # host threads stepping the chains (0: one for every four chains, at
    # most 8; 1: the calling thread); the results are the same for every
    # value
    host_threads: int = 0


LAUNCH = {"streams": 0, "batch": 1, "independent": 2}


def _config(settings: McmcSettings) -> "nat.McmcConfig":
    w = np.zeros(nat.OP_COUNT)
    for name, val in settings.weights.items():
        w[OPERATORS.index(name)] = val
    return nat.McmcConfig(settings.num_chains, settings.num_categories,
                          nat.PRECISION_F64 if settings.precision == "f64"
                          else nat.PRECISION_F32,
                          MODELS[settings.model], settings.seed, settings.heat,
                          settings.swap_every, settings.sample_every, settings.tune_every,
                          settings.device, (ct.c_double * nat.OP_COUNT)(*w),
                          settings.da_pilot_steps, settings.da_epochs, settings.da_hidden,
                          0, settings.da_drift_limit, settings.clock_categories,
                          LAUNCH[settings.launch], settings.host_threads)


class Mcmc:
    def __init__(self, leaves: np.ndarray, weights: np.ndarray, parents: np.ndarray,
                 heights: np.ndarray, settings: McmcSettings):
        leaves = nat.u8(leaves)
        L, P = leaves.shape
        cfg = _config(settings)
        self._wts = nat.u32(weights)
        self._par = nat.u32(parents)
        self._hei = nat.f64(heights)
        h = ct.c_void_p()
        check(lib.b3g_mcmc_create(ct.byref(cfg), L, P, nat.as_ptr(leaves, ct.c_uint8),
                                  nat.as_ptr(self._wts, ct.c_uint32),
                                  nat.as_ptr(self._par, ct.c_uint32),
                                  nat.as_ptr(self._hei, ct.c_double), ct.byref(h)))
        self._h = h
        self.settings = settings
        self.num_nodes = self._par.size
        self.chain_nodes = [self.num_nodes] * settings.num_chains

    @classmethod
    def multi(cls, problems, settings: McmcSettings) -> "Mcmc":
        """Chains over several alignments (b3g_mcmc_create_multi):
        `problems` is a list of (leaves, weights, parents, heights);
        settings.num_chains / len(problems) chains per problem form that
        problem's temperature ladder (MC3 swaps within a problem only)."""
        self = cls.__new__(cls)
        self._keep = []
        arr = (nat.McmcProblem * len(problems))()
        for k, (leaves, weights, parents, heights) in enumerate(problems):
            lv, wt = nat.u8(leaves), nat.u32(weights)
            pa, he = nat.u32(parents), nat.f64(heights)
            self._keep += [lv, wt, pa, he]
            arr[k] = nat.McmcProblem(lv.shape[0], lv.shape[1], lv.ctypes.data,
                                     wt.ctypes.data, pa.ctypes.data, he.ctypes.data)
        h = ct.c_void_p()
        check(lib.b3g_mcmc_create_multi(ct.byref(_config(settings)), len(problems), arr,
                                        ct.byref(h)))
        self._h = h
        self.settings = settings
        group = settings.num_chains // len(problems)
        sizes = [nat.u32(p[2]).size for p in problems]
        self.chain_nodes = [sizes[i // group] for i in range(settings.num_chains)]
        self.num_nodes = sizes[0]
        return self

    def launch_stats(self) -> dict:
        """{"batched": launch mode is the batched graph, "device_ms": device
        time of its replays so far, "launches": their count}."""
        b, ms, n = ct.c_uint32(), ct.c_double(), ct.c_uint64()
        check(lib.b3g_mcmc_launch_stats(self._h, ct.byref(b), ct.byref(ms), ct.byref(n)))
        return {"batched": bool(b.value), "device_ms": ms.value, "launches": n.value}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib.b3g_mcmc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_parameters(self, kappa=2.0, rates=None, frequencies=None, alpha=0.5,
                       birth_rate=1.0):
        r = None if rates is None else nat.f64(rates)
        f = None if frequencies is None else nat.f64(frequencies)
        check(lib.b3g_mcmc_set_parameters(
            self._h, float(kappa), None if r is None else nat.as_ptr(r, ct.c_double),
            None if f is None else nat.as_ptr(f, ct.c_double), float(alpha),
            float(birth_rate)))

    def set_clock(self, sd: float, categories=None):
        """Relaxed-clock start state (before ``set_parameters``): the LogNormal
        sd and one category per node (its parent edge; the root's is
        ignored), or None for node % k."""
        c = None if categories is None else nat.u32(categories)
        check(lib.b3g_mcmc_set_clock(self._h, float(sd),
                                     None if c is None else nat.as_ptr(c, ct.c_uint32)))

    def run(self, steps: int):
        check(lib.b3g_mcmc_run(self._h, int(steps)))

    def trace(self, name: str, chain: int | None = None) -> np.ndarray:
        """Samples of one trace field: the cold chain's, or chain `chain`'s
        (chain order; independent replicates when heat = 0)."""
        fid = TRACE_FIELDS.index(name)
        n = ct.c_uint64()
        if chain is None:
            check(lib.b3g_mcmc_trace(self._h, fid, None, 0, ct.byref(n)))
            out = np.empty(n.value)
            check(lib.b3g_mcmc_trace(self._h, fid, nat.as_ptr(out, ct.c_double), n.value,
                                     ct.byref(n)))
            return out
        check(lib.b3g_mcmc_chain_trace(self._h, int(chain), fid, None, 0, ct.byref(n)))
        out = np.empty(n.value)
        check(lib.b3g_mcmc_chain_trace(self._h, int(chain), fid,
                                       nat.as_ptr(out, ct.c_double), n.value, ct.byref(n)))
        return out

    def samples(self) -> dict:
        """Every sample of the cold chain: steps, tree (parents and heights of
        every node) and parameters."""
        n = ct.c_uint64()
        check(lib.b3g_mcmc_samples(self._h, None, None, None, None, 0, ct.byref(n)))
        k = n.value
        steps = np.zeros(k, dtype=np.uint64)
        parents = np.zeros((k, self.num_nodes), dtype=np.uint32)
        heights = np.zeros((k, self.num_nodes))
        params = np.zeros((k, 14))
        check(lib.b3g_mcmc_samples(
            self._h, steps.ctypes.data_as(ct.POINTER(ct.c_uint64)),
            nat.as_ptr(parents, ct.c_uint32), nat.as_ptr(heights, ct.c_double),
            nat.as_ptr(params, ct.c_double), k, ct.byref(n)))
        return {"step": steps, "parents": parents, "heights": heights,
                "kappa": params[:, 0], "alpha": params[:, 1], "birth_rate": params[:, 2],
                "rates": params[:, 3:9], "frequencies": params[:, 9:13],
                "clock_sd": params[:, 13]}

    def operator_stats(self) -> dict:
        out = {}
        for k, name in enumerate(OPERATORS):
            counts = (ct.c_uint64 * 4)()
            tuning = ct.c_double()
            check(lib.b3g_mcmc_operator_stats(self._h, k, counts, ct.byref(tuning)))
            out[name] = dict(accepts=counts[0], rejects=counts[1], aborts=counts[2],
                             prior_rejects=counts[3], tuning=tuning.value)
        return out

    def set_tuning(self, tunings: dict) -> None:
        """Start values of operators' tuning parameters by name (e.g. the
        ``tuning`` entries of another run's ``operator_stats``)."""
        for name, value in tunings.items():
            check(lib.b3g_mcmc_set_tuning(self._h, OPERATORS.index(name), float(value)))

    def swaps(self) -> tuple[int, int]:
        t, a = ct.c_uint64(), ct.c_uint64()
        check(lib.b3g_mcmc_swaps(self._h, ct.byref(t), ct.byref(a)))
        return t.value, a.value

    def da_stats(self) -> dict:
        counts = (ct.c_uint64 * 6)()
        values = (ct.c_double * 2)()
        check(lib.b3g_mcmc_da_stats(self._h, counts, values))
        keys = ["pilot_pairs", "stage1_rejects", "stage2_accepts", "stage2_rejects",
                "exact_evaluations", "fallback"]
        out = {k: int(v) for k, v in zip(keys, counts)}
        out["train_loss"], out["drift_rms"] = values[0], values[1]
        return out

    def dump(self) -> bytes:
        """Checkpoint of the driver between runs (b3g_mcmc_dump)."""
        size = ct.c_uint64()
        check(lib.b3g_mcmc_dump(self._h, None, 0, ct.byref(size)))
        buf = np.empty(size.value, dtype=np.uint8)
        check(lib.b3g_mcmc_dump(self._h, nat.as_ptr(buf, ct.c_uint8), size.value,
                                ct.byref(size)))
        return buf.tobytes()

    def load(self, state: bytes) -> None:
        """Continue from a checkpoint of a driver with the same
        configuration and data (b3g_mcmc_load); traces start empty."""
        buf = np.frombuffer(state, dtype=np.uint8)
        check(lib.b3g_mcmc_load(self._h, nat.as_ptr(np.ascontiguousarray(buf), ct.c_uint8),
                                buf.size))

    @staticmethod
    def _state_layout(parameters, operators):
        params = nat.u32([STATE_PARAMETERS.index(p) for p in parameters])
        ops = nat.u32([[OPERATORS.index(name), int(bool(tuned))]
                       for name, tuned in operators]).reshape(-1)
        return params, ops

    def dump_verbatim(self, parameters, operators, chain: int = 0) -> bytes:
        """One chain's state in the reference's state-file layout
        (b3g_mcmc_dump_verbatim): `parameters` in the reference Mcmc's
        order (names of STATE_PARAMETERS), `operators` in its scheduler's
        order as (OPERATORS name, has a tuning) pairs."""
        params, ops = self._state_layout(parameters, operators)
        size = ct.c_uint64()
        args = (self._h, chain, nat.as_ptr(params, ct.c_uint32), params.size,
                nat.as_ptr(ops, ct.c_uint32), ops.size // 2)
        check(lib.b3g_mcmc_dump_verbatim(*args, None, 0, ct.byref(size)))
        buf = np.empty(size.value, dtype=np.uint8)
        check(lib.b3g_mcmc_dump_verbatim(*args, nat.as_ptr(buf, ct.c_uint8), size.value,
                                         ct.byref(size)))
        return buf.tobytes()

    def load_verbatim(self, state: bytes, parameters, operators, chain: int = 0) -> None:
        """Take a state in the reference's layout into one chain (and the
        driver's step and operator statistics), re-evaluating it
        (b3g_mcmc_load_verbatim)."""
        params, ops = self._state_layout(parameters, operators)
        buf = np.ascontiguousarray(np.frombuffer(state, dtype=np.uint8))
        check(lib.b3g_mcmc_load_verbatim(self._h, chain, nat.as_ptr(params, ct.c_uint32),
                                         params.size, nat.as_ptr(ops, ct.c_uint32),
                                         ops.size // 2, nat.as_ptr(buf, ct.c_uint8),
                                         buf.size))

    def check(self) -> float:
        out = ct.c_double()
        check(lib.b3g_mcmc_check(self._h, ct.byref(out)))
        return out.value

    def chain_state(self, chain: int):
        parents = np.zeros(self.chain_nodes[chain], dtype=np.uint32)
        heights = np.zeros(self.chain_nodes[chain])
        lnl, beta = ct.c_double(), ct.c_double()
        check(lib.b3g_mcmc_chain_state(self._h, chain, nat.as_ptr(parents, ct.c_uint32),
                                       nat.as_ptr(heights, ct.c_double), ct.byref(lnl),
                                       ct.byref(beta)))
        return parents, heights, lnl.value, beta.value
