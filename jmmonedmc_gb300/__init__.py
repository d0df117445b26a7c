"""jmmOneDMC's Monte Carlo move loop on one GB300 (sm_103a).

The product is libjmmgpu.so (include/jmm_gpu.h), built in-tree by
``jmmonedmc_gb300.build``; this package holds its ctypes mirror and the
Python handles used by scripts, tests and the benchmark:

- ``plain.PlainChain``   one FP64 chain, the reference's algorithm step for step
                         (``python -m jmmonedmc_gb300.plain`` times it)
- ``batch.ChainBatch``   thousands of independent chains in one persistent kernel,
                         with sampled rho(x)/g(x) histograms and checkpoints
- ``large.LargeChains``  chains of up to 2^24 particles (alternating-domain sweep)
- ``grad``               energy gradients w.r.t. (eps, sigma, L) for torch
- ``inputfile``, ``thermo``  the reference's INPUT keywords and output line formats

The C++ drop-in for the reference's MCState API lives in ``dropin/``.
"""
__version__ = "0.1.0"
