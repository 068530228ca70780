"""CPU tests of the C ABI: the shared library builds for sm_103a, loads, and
exports every function include/lcf.h declares (no GPU call is made)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "lcf.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:int|void|const char\*|void\*)\s+\**(\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="session")
def libpath():
    from lightcurve_fitting_gb300 import build
    return build.build()


# every symbol the reference's Rust host declares in its extern blocks
# (src/gpu_cuda.rs:17-164)
REFERENCE_FFI = ["launch_bazin", "launch_villar", "launch_tde", "launch_arnett", "launch_magnetar",
                 "launch_shock_cooling", "launch_afterglow", "launch_metzger_kn", "launch_batch_pso_cost",
                 "launch_batch_pso_cost_multi_bazin", "launch_batch_svi_fit"]


def test_header_declares_the_reference_exports():
    names = declared_functions()
    for n in REFERENCE_FFI + ["lcf_ctx_create", "lcf_fit_parametric_batch", "lcf_band_cost"]:
        assert n in names


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_context_creation_fails_cleanly_without_gpu(libpath):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from lightcurve_fitting_gb300.lib import Context, LcfError
    with pytest.raises(LcfError):
        Context(0)


def test_python_api_validates_arguments():
    from lightcurve_fitting_gb300 import parametric
    with pytest.raises(ValueError, match="bogus"):
        parametric._method("bogus")
    with pytest.raises(ValueError):
        parametric._model_id("NotAModel")
    assert parametric._model_id("tde") == 2


def test_build_flux_bands_matches_reference_rules():
    from lightcurve_fitting_gb300.parametric import build_flux_bands
    import numpy as np
    t = [2460000.0, 2460001.0, 2460002.0, 2460003.0]
    m = [20.0, float("nan"), 19.0, 21.0]
    e = [0.1, 0.1, 0.1, 0.2]
    b = ["g", "g", "r", "g"]
    out = build_flux_bands(t, m, e, b)
    assert sorted(out) == ["g", "r"]
    assert out["g"]["times"] == [0.0, 3.0]
    np.testing.assert_allclose(out["r"]["values"][0], 10 ** (-0.4 * (19.0 - 23.9)))


def test_struct_layouts_match_the_ctypes_mirror(tmp_path):
    """Every struct of include/lcf.h, compiled by the C compiler, has the size
    and field offsets of its ctypes Structure in abi.py."""
    import subprocess
    from lightcurve_fitting_gb300 import abi
    pairs = {"lcf_bands_csr": abi.BandsCSR, "lcf_fit_options": abi.FitOptions, "lcf_fit_outputs": abi.FitOutputs,
             "lcf_fit_stats": abi.FitStats, "lcf_pso_selection": abi.PsoSelection}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "lcf.h"', "int main(void) {"]
    for cname, cls in pairs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = {}
    for row in subprocess.check_output([str(exe)]).decode().split("\n"):
        if row:
            cname, field, v = row.split()
            got[(cname, field)] = int(v)
    for cname, cls in pairs.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


def test_rust_bindings_in_the_integration_notes_match_the_header():
    """A documentation-sync test: the #[repr(C)] structs a maintainer adds to
    the Rust crate (written out in INTEGRATION.md, which this test reads)
    list the header's fields in the header's order."""
    from lightcurve_fitting_gb300 import abi
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    pairs = {"LcfBandsCsr": abi.BandsCSR, "LcfFitOptions": abi.FitOptions, "LcfFitOutputs": abi.FitOutputs,
             "LcfPsoSelection": abi.PsoSelection}
    for rname, cls in pairs.items():
        m = re.search(r"pub struct " + rname + r"\s*\{(.*?)\}", text, flags=re.S)
        assert m, rname
        fields = re.findall(r"pub (\w+)\s*:", m.group(1))
        assert fields == [f for f, _ in cls._fields_], rname


def test_build_raw_flux_bands_matches_reference_rules():
    """build_raw_flux_bands (src/common.rs:117-149): times relative to the
    earliest time of all rows (dropped rows included), non-finite or
    non-positive fluxes and errors dropped, linear values kept."""
    from lightcurve_fitting_gb300.parametric import build_raw_flux_bands
    t = [10.0, 11.0, 12.0, 13.0, 14.0]
    f = [5.0, -1.0, 7.0, float("nan"), 2.0]
    e = [0.5, 0.5, 0.0, 0.5, 0.25]
    b = ["g", "g", "r", "r", "r"]
    out = build_raw_flux_bands(t, f, e, b)
    assert out == {"g": {"times": [0.0], "values": [5.0], "errors": [0.5]},
                   "r": {"times": [4.0], "values": [2.0], "errors": [0.25]}}
    assert build_raw_flux_bands([], [], [], []) == {}


def test_python_api_rejects_before_touching_the_gpu():
    from lightcurve_fitting_gb300 import parametric
    with pytest.raises(ValueError, match="two non-empty bands"):
        parametric.fit_parametric_multiband({"g": {"times": [0.0], "values": [1.0], "errors": [0.1]},
                                             "r": {"times": [], "values": [], "errors": []}})
    assert parametric.fit_parametric_multiband({}) == []
    with pytest.raises(ValueError, match="takes 6 parameters"):
        parametric.eval_model("Bazin", [0.0, 0.1], [1.0])
    with pytest.raises(ValueError):
        parametric.eval_model("NoSuchModel", [0.0], [1.0])
