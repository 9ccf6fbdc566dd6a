"""mczi_gb300 -- the MC/ZI k-mer hot path on one GB300 (sm_103a).

The kernels and the C ABI live in ``lib/libmczi_gpu.so`` (sources in
``csrc/``, header ``include/mczi_gpu.h``); this package is the host-side
mirror of the reference's library interface:

* :mod:`mczi_gb300.mc` -- MC counting (``count_inputs``, ``count_datasets``,
  ``count_*_to_kff_path``, ``count_*_to_fasta_path``)
* :mod:`mczi_gb300.gen` -- seeded synthetic workloads
* :mod:`mczi_gb300.build` -- in-tree build of the native libraries
"""
from ._native import MCZIError, MODE_ABUNDANCE, MODE_PRESENCE  # noqa: F401

__all__ = ["MCZIError", "MODE_ABUNDANCE", "MODE_PRESENCE"]
