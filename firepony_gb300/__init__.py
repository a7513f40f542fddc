"""firepony_gb300 — a GB300-native (sm_103a) BQSR engine behind Firepony's pipeline seam.

The hot path (read filters, CIGAR expansion, known-site filter, BAQ, fractional errors, covariate keys,
sort/reduce into the covariate tables, empirical quality) runs as hand-written CUDA kernels in
``_build/libfpengine.so``; its C ABI is ``include/firepony_gb300.h``. This package holds the in-tree build
(:mod:`firepony_gb300.build`), the Python binding of the C ABI (:mod:`firepony_gb300.engine`) and the
seeded synthetic-input generator (:mod:`firepony_gb300.synth`).
"""

__all__ = ["build", "engine", "synth", "abi"]
