"""CPU oracle for the lens image-simulation path (TEST INFRASTRUCTURE ONLY).

This package is a NumPy/SciPy FP64 restatement of JAXtronomy's
``ImageModel.image`` path (ray shooting -> surface brightness -> supersampling ->
PSF convolution -> re-binning) and of its image log-likelihood.  Each function
cites the reference file:line it follows (paths are relative to the JAXtronomy
source tree).

It exists only to *check* the CUDA implementation in ``jaxtronomy_gb300``:
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
may import it; product code must never import or call it, and there is no CPU
fallback through it.

Parity status
-------------
* Pinned: the JAXtronomy-owned formulas (lens/light profiles, numerics,
  convolution, likelihood) are checked against golden vectors produced by running
  the reference's own source under a NumPy-backed stand-in for ``jax``
  (``tests/golden/make_golden.py``), and ``hyp2f1_lopez_temme_8`` against
  ``scipy.special.hyp2f1`` at the reference test points.
* Unpinned: conventions that the reference imports from the un-vendored
  ``lenstronomy`` package (pixel-grid and supersampled-grid construction,
  ``Image2SourceMapping``, the PSF class) are restated here from lenstronomy's
  published behaviour; the reference tests that would pin them compare against a
  live lenstronomy install, which is not available.
"""

from . import grid, lens, light, numerics, image  # noqa: F401

__all__ = ["grid", "lens", "light", "numerics", "image"]
