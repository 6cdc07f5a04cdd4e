"""aspartik_gb300 -- GB300 (sm_103a) Felsenstein-pruning likelihood for b3.

A drop-in for the likelihood path of the b3 MCMC engine of
kaathewisegit/aspartik.  The compute path is ``libb3g.so`` (hand-written
CUDA for sm_103a behind the C ABI in ``include/b3g.h``); this package holds
its Python face, the build recipe and the synthetic-data simulators.

Submodules are imported lazily so that ``aspartik_gb300.build`` works before
the library exists.
"""

__version__ = "0.1.0"
