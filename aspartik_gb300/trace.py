"""Trace files in the layout of the reference's TraceWriter
(crates/b3/src/callback/trace_writer.rs:166-492): one Arrow IPC file, one
row per sample, non-nullable columns `step` (u64), `posterior`, `prior`,
`likelihood` (f64), then per logged item a column named after it (a real:
f64; a vector: fixed-size list of f64) and for the tree the four columns
`tree:parents` (fixed-size list of u32, one per node, root 0xFFFFFFFF),
`tree:heights` (fixed-size list of f64), `tree:length` and `tree:height`
(f64); schema metadata `aspartik`, `os`, `arch`, `time`.  The reference's
replicate tooling reads trees back from the `:parents`/`:heights` columns.

Written with pyarrow (host side, after the run); the samples come from the
native driver (`Mcmc.samples`, `Mcmc.trace`).
"""

from __future__ import annotations

import platform
import time

import numpy as np

from . import __version__


def _fixed(values: np.ndarray, pa_type):
    import pyarrow as pa

    n, k = values.shape
    flat = pa.array(values.reshape(-1), type=pa_type)
    return pa.FixedSizeListArray.from_arrays(flat, k)


def write_trace(path, mcmc, tree_name: str = "tree", zstd: bool = False) -> int:
    """Write every sample of `mcmc`'s cold chain; returns the row count."""
    import pyarrow as pa
    import pyarrow.ipc as ipc

    smp = mcmc.samples()
    n = smp["step"].size
    lnl = mcmc.trace("lnl")[:n]
    prior = mcmc.trace("prior")[:n]
    parents, heights = smp["parents"], smp["heights"]
    roots = np.argmax(parents == 0xFFFFFFFF, axis=1)
    root_height = heights[np.arange(n), roots]
    with np.errstate(invalid="ignore"):
        par_h = np.where(parents == 0xFFFFFFFF, 0.0,
                         np.take_along_axis(heights, np.minimum(parents, parents.shape[1] - 1)
                                            .astype(np.int64), axis=1))
    length = np.where(parents == 0xFFFFFFFF, 0.0, par_h - heights).sum(axis=1)
    cols = {
        "step": pa.array(smp["step"], type=pa.uint64()),
        "posterior": pa.array(lnl + prior, type=pa.float64()),
        "prior": pa.array(prior, type=pa.float64()),
        "likelihood": pa.array(lnl, type=pa.float64()),
        "birth_rate": pa.array(smp["birth_rate"], type=pa.float64()),
        "alpha": pa.array(smp["alpha"], type=pa.float64()),
    }
    if mcmc.settings.model == "hky":
        cols["kappa"] = pa.array(smp["kappa"], type=pa.float64())
    else:
        cols["rates"] = _fixed(smp["rates"], pa.float64())
    cols["frequencies"] = _fixed(smp["frequencies"], pa.float64())
    if mcmc.settings.clock_categories:
        cols["clock_sd"] = pa.array(smp["clock_sd"], type=pa.float64())
    cols[f"{tree_name}:parents"] = _fixed(parents, pa.uint32())
    cols[f"{tree_name}:heights"] = _fixed(heights, pa.float64())
    cols[f"{tree_name}:length"] = pa.array(length, type=pa.float64())
    cols[f"{tree_name}:height"] = pa.array(root_height, type=pa.float64())
    fields = [pa.field(k, v.type, nullable=False) for k, v in cols.items()]
    meta = {"aspartik": f"aspartik_gb300 {__version__}", "os": platform.system().lower(),
            "arch": platform.machine(), "time": str(int(time.time()))}
    schema = pa.schema(fields, metadata=meta)
    table = pa.Table.from_arrays(list(cols.values()), schema=schema)
    opts = ipc.IpcWriteOptions(compression="zstd" if zstd else None)
    with ipc.new_file(str(path), schema, options=opts) as w:
        w.write_table(table)
    return n


def read_trees(path, tree_name: str = "tree"):
    """(parents [n][nodes], heights [n][nodes]) from a trace file."""
    import pyarrow.ipc as ipc

    table = ipc.open_file(str(path)).read_all()
    par = table[f"{tree_name}:parents"].combine_chunks()
    hei = table[f"{tree_name}:heights"].combine_chunks()
    k = par.type.list_size
    return (np.asarray(par.values).reshape(-1, k).astype(np.uint32),
            np.asarray(hei.values).reshape(-1, k))
