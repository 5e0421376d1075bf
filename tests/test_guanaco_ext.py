"""The drop-in module guanaco_ext (CPU): it exports every name of the
reference's extension module, and the reference's own Python package, when it
is present (the directory named by GUANACO_REFERENCE, or a "reference"
directory beside this repository), imports it as its native layer and gets
this library's functions and CTF known answers."""
import importlib
import os
import sys
import types

import numpy as np
import pytest

from conftest import REPO, golden

NAMES = ["eDevice", "cpu", "gpu", "recon", "corr", "CTF", "get_electron_wavelength",
         "get_defocus_spread", "q_to_Q", "Q_to_q", "df_to_D", "D_to_df", "get_q_and_theta"]


def test_module_exports_the_reference_names():
    import guanaco_ext

    for name in NAMES:
        assert hasattr(guanaco_ext, name), name
    assert sorted(guanaco_ext.__all__) == sorted(NAMES)
    assert guanaco_ext.eDevice.convert("gpu") == guanaco_ext.gpu


def _reference_src():
    root = os.environ.get("GUANACO_REFERENCE") or os.path.join(os.path.dirname(REPO),
                                                                 "reference")
    src = os.path.join(root, "src")
    return src if os.path.isdir(os.path.join(src, "guanaco")) else None


def test_reference_package_runs_on_this_module():
    src = _reference_src()
    if src is None:
        pytest.skip("the reference's source tree is not on this machine")
    saved = {k: sys.modules.pop(k) for k in list(sys.modules)
             if k == "guanaco" or k.startswith("guanaco.") or k == "guanaco_ext"}
    sys.path.insert(0, src)
    sys.path.insert(0, REPO)  # this repository's guanaco_ext first
    stub = "mrcfile" not in sys.modules
    if stub:  # the reference's file readers import mrcfile; not needed here
        sys.modules["mrcfile"] = types.ModuleType("mrcfile")
    try:
        guanaco = importlib.import_module("guanaco")
        import guanaco_gb300.detail as D

        assert guanaco.detail.recon is D.recon and guanaco.detail.corr is D.corr
        g = golden("ctf_kat")
        l = guanaco.detail.get_electron_wavelength(300000)
        assert l == pytest.approx(float(g["wavelength_300kV"]), rel=1e-15)
        ctf = guanaco.detail.CTF(l, 20000, 2.7e7)
        assert ctf.get_chi(10, 0) == pytest.approx(float(g["chi_q10"]), rel=1e-15)
        # the reference's own CTF stack (correct.py:157-214) through this
        # module's CTF class, against the oracle's restatement
        from oracle import oracle as O

        arr = guanaco.detail.correct.get_ctf_array(24, 16, 1.0, 300, 20000.0, 3, 500.0, 2.7)
        want = O.ctf_stack(24, 16, 1.0, 300, 20000.0, 3, 500.0, 2.7)
        assert arr.shape == (3, 16, 24)
        np.testing.assert_array_equal(arr.astype(np.complex64), want)
    finally:
        sys.path.remove(src)
        sys.path.remove(REPO)
        for k in [k for k in sys.modules if k == "guanaco" or k.startswith("guanaco.")
                  or k == "guanaco_ext"]:
            sys.modules.pop(k)
        if stub:
            sys.modules.pop("mrcfile", None)
        sys.modules.update(saved)
