"""guanaco_gb300: guanaco's 3D-CTF filtered-backprojection path on GB300
(sm_103a), behind the reference's own interfaces.

* ``guanaco_gb300.detail`` -- drop-in for the pybind11 module ``guanaco_ext``
  (``recon``, ``corr``, ``CTF``, ``eDevice`` ...).
* ``correct_projections`` / ``reconstruct`` -- drop-ins for the public
  ``guanaco`` functions on the device path; ``reconstruct_ctf`` runs both in
  one device pass.
* ``FbpPlan`` -- the whole-series plan over the C ABI (include/guanaco_gb300.h).
* ``reconstruct_file`` / ``correct_file`` -- the MRC file entry points
  (``guanaco_gb300.mrc`` reads and writes MRC2014 with FEI1 headers).
* ``serve.Server`` -- the request server: many tilt series of mixed shapes at
  once, with continuous batching on one GPU.
* ``plot.generate_ctf`` -- the CTF images of a defocus series, computed on the
  GPU and written as a complex64 MRC stack.
"""
from . import detail  # noqa: F401
from .api import (  # noqa: F401
    compute_angular_weights,
    correct_projections,
    get_centre,
    get_ctf,
    get_ctf_array,
    get_defocus_steps,
    get_weights,
    correct_file,
    reconstruct,
    reconstruct_ctf,
    reconstruct_file,
)
from .fbp import FbpDesc, FbpPlan  # noqa: F401
from . import plot  # noqa: F401

__version__ = "0.1.0"
