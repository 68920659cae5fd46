"""The drop-in multigrid module libamrd_mg_gb300 without a GPU: it exports
the reference's amrd/mg.c entry points (amrd/mg.h:32-37 and the cmask
helpers evolve.c and cls.c call), links into the reference's own AMRD in
place of amrd/mg.o, and the test application builds against it; without a
GPU a solve stops with a message instead of computing anything on the host.
"""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "dropin"))
import dropin as D  # noqa: E402
import golden_cases as G  # noqa: E402
from oracle import refrun  # noqa: E402
from pamr_amrd_gb300 import build as B  # noqa: E402

REFERENCE_ENTRY_POINTS = {"solve_elliptics", "vcycle", "set_cmask_bdy", "extend_cmask_bdy"}
ADDITIONS = {"amrd_set_device_MG_operator", "amrd_set_device_MG_precision", "amrd_device_MG_residuals",
             "amrd_device_MG_release"}


def _dynsyms(path, defined=True):
    nm = shutil.which("nm")
    if not nm:
        pytest.skip("nm not available")
    flag = "--defined-only" if defined else "--undefined-only"
    out = subprocess.run([nm, "-D", flag, path], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


def test_exports_the_reference_entry_points():
    B.build()
    syms = _dynsyms(B.LIB_AMRD_MG)
    assert REFERENCE_ENTRY_POINTS <= syms
    assert ADDITIONS <= syms
    # everything else it needs comes from the application's PAMR / AMRD
    und = _dynsyms(B.LIB_AMRD_MG, defined=False)
    assert {"PAMR_get_sgh", "PAMR_get_g_attribs", "PAMR_get_gfn", "AMRD_MG_tol", "AMRD_stop"} <= und


@pytest.mark.skipif(not refrun.available(), reason="reference sources not built here")
def test_links_into_the_reference_amrd_in_place_of_mg_o():
    """oracle/build_ref.sh links the application against the reference's
    PAMR/AMRD objects without amrd/mg.o plus libamrd_mg_gb300.a: every
    symbol evolve.c and cls.c take from mg.c resolves"""
    assert os.path.exists(D.LINK_CHECK_APP)


def test_device_application_builds():
    assert os.path.exists(D.build_device_app())


def test_reference_application_matches_the_fixtures():
    """the reference build of the application reproduces its fixtures (the
    application and its reference environment are deterministic)"""
    if not os.path.exists(D.REF_APP):
        pytest.skip("reference sources not built here")
    for path in G.dropin_files()[:2]:
        case, mode, arg, level, ref = G.load_dropin(path)
        out = D.run(D.REF_APP, case, mode, arg, level)
        assert out["iters"] == ref["iters"]
        for a, b in zip(out["grids"], ref["grids"]):
            assert np.array_equal(a["u"], b["u"]) and np.array_equal(a["cmask"], b["cmask"])


def test_without_a_gpu_the_solve_stops_with_a_message():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    case, mode, arg, level, _ = G.load_dropin(G.dropin_files()[0])
    with pytest.raises(RuntimeError) as e:
        D.run(D.build_device_app(), case, mode, arg, level)
    assert "libamrd_mg_gb300" in str(e.value)
