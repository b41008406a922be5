"""LF_DEM itself built with the GB300 engine behind its StokesSolver: every
LF_DEM source except StokesSolver.cpp, compiled unmodified from the directory
that LFDEM_REF names, plus lf_dem_gb300/adapter/StokesSolverGB300.cpp, linked
to liblfdem_gb300.so (lf_dem_gb300/adapter/Makefile).  Compile and link only:
the test needs no GPU, and it is skipped where LFDEM_REF is not set."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(ROOT, "lf_dem_gb300", "adapter")


@pytest.fixture(scope="module")
def ref_dir():
    ref = os.environ.get("LFDEM_REF")
    if not ref or not os.path.isfile(os.path.join(ref, "StokesSolver.h")):
        pytest.skip("LFDEM_REF does not name LF_DEM's source directory")
    return ref


def test_lfdem_links_against_the_engine(ref_dir):
    from lf_dem_gb300 import build as B
    B.build()
    out = subprocess.run(["make", "-C", ADAPTER, f"LFDEM_REF={ref_dir}", "-j8", "all", "check-link"],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stdout[-3000:] + out.stderr[-3000:]
    exe = os.path.join(ADAPTER, "_build", "LF_DEM_gb300")
    assert os.access(exe, os.X_OK)
    # every StokesSolver symbol LF_DEM calls comes from the adapter, and the
    # adapter's own references all resolve in liblfdem_gb300.so
    nm = subprocess.run(["nm", "-C", "--defined-only", os.path.join(ADAPTER, "_build", "StokesSolverGB300.o")],
                        capture_output=True, text=True).stdout
    for sym in ("StokesSolver::init", "StokesSolver::resetResistanceMatrix", "StokesSolver::addResistanceBlocks",
                "StokesSolver::matrixFillingDone", "StokesSolver::solve", "StokesSolver::compute_LTRHS"):
        assert sym in nm, sym
    ldd = subprocess.run(["ldd", exe], capture_output=True, text=True).stdout
    assert "liblfdem_gb300.so" in ldd
