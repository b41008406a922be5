"""The ctypes mirrors of the C ABI's structs (lf_dem_gb300/__init__.py)
against include/lfdem_gb300.h: a small C program compiled with the host
compiler prints every struct's size and each field's offset, which must equal
the ctypes layout (a mismatch would make a call write past a Python buffer)."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

import lf_dem_gb300 as E

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PAIRS = [(E.Status, "lfg_status"), (E.OutputUnits, "lfg_output_units"), (E.OutputConfig, "lfg_output_config"),
         (E.Params, "lfg_params"), (E.Options, "lfg_options"), (E.SolverStats, "lfg_solver_stats"),
         (E.SimScalars, "lfg_sim_scalars"), (E.Pair, "lfg_pair"), (E.Request, "lfg_request"),
         (E.Result, "lfg_result"), (E.ServerStats, "lfg_server_stats"), (E.BatchStats, "lfg_batch_stats"),
         (E.SimTiming, "lfg_sim_timing")]


def _c_has_field(cname, name):
    with open(os.path.join(ROOT, "include", "lfdem_gb300.h")) as f:
        hdr = f.read()
    end = hdr.find("} " + cname + ";")
    start = hdr.rfind("typedef struct", 0, end)
    body = hdr[start:end]
    return any(tok.strip(" ;\t[]0123456789") == name for line in body.split("\n") for tok in line.split())


def test_struct_layouts_match_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "lfdem_gb300.h"', "int main(void) {"]
    expect = []
    for cls, cname in PAIRS:
        lines.append(f'printf("%zu\\n", sizeof({cname}));')
        expect.append((cname, "sizeof", C.sizeof(cls)))
        for f in cls._fields_:
            name = f[0]
            if name.startswith("pad") and name.endswith("_") and not _c_has_field(cname, name):
                continue   # explicit ctypes padding where C pads implicitly
            lines.append(f'printf("%zu\\n", offsetof({cname}, {name}));')
            expect.append((cname, name, getattr(cls, name).offset))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert len(got) == len(expect)
    bad = [(c, n, e, g) for (c, n, e), g in zip(expect, got) if e != g]
    assert not bad, bad
