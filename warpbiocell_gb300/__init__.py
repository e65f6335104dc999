"""warpbiocell_gb300: WarpBioCell's coupled cell step on GB300 (sm_103a).

A drop-in for the reference's model APIs (``warpbiocell.cells``, ``.spatial``, ``.fields``,
``.network``, ``.simulation.simulator``): the same module layout, classes and signatures, with
torch CUDA tensors as the arrays and hand-written CUDA kernels behind the C-ABI in
``include/wbc.h`` (libwbc_gb300.so). There is no CPU fallback.

Units as in the reference: lengths in um, times in h.
"""

__version__ = "0.1.0"
