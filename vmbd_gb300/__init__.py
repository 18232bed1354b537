"""GB300-native efficient-filter-flow (EFF) operator for VMBD-style
spatially varying blind deconvolution.

The hot path -- OlaGPU's forward operator, its two adjoints and the PSF
projections -- runs as hand-written sm_103a CUDA kernels behind the C ABI in
``include/vmbd_eff.h`` (``vmbd_gb300/_lib/libvmbd_eff.so``).  Python mirrors
the reference's interface: ``win2winaux``, ``OlaGPU`` (``cnv``/``cnvtp``),
the ``gputools`` projections and the ``PBB`` optimiser, plus a
``torch.autograd.Function`` (``eff``).
"""
from .geometry import Winaux, win2winaux, patch_geometry, fft_frame  # noqa: F401
from . import synth  # noqa: F401


def __getattr__(name):
    # torch-dependent parts load lazily so that geometry/synth work without CUDA.
    if name in ("EffPlan", "project_psf", "basis_project"):
        from . import eff
        return getattr(eff, name)
    if name in ("EFFFunction", "eff"):
        from . import autograd
        return getattr(autograd, name)
    if name == "OlaGPU":
        from .olagpu import OlaGPU
        return OlaGPU
    raise AttributeError(name)
