"""The drop-in integration recipe, checked on the CPU: a temporary copy of the reference's
Limit-sticky9.c with a PN_GPU guard around its own force/energy functions compiles with gcc and
its main loop links against libpn's drop-in entry points (run only where the reference source
is present; the linked binary itself runs on the GPU in test_reference_main_gpu.py)."""
import os
import subprocess

import pytest

from conftest import ROOT
from oracle import pyoracle

LS9 = os.path.join(pyoracle.reference_dir(), "Limit-sticky9.c")


@pytest.mark.skipif(not os.path.exists(LS9), reason="reference source not present")
def test_reference_main_links_against_libpn(tmp_path):
    lines = open(LS9).read().split("\n")
    # Limit-sticky9.c:15 is '#pragma goose func' (before rsqrt); :738 closes push_position
    assert lines[14].startswith("#pragma goose func")
    assert lines[737].strip() == "}" and "push_position" in "\n".join(lines[727:730])
    patched = (lines[:14] + ["#ifdef PN_GPU", '#include "pn.h"', "#else"] + lines[14:738]
               + ["#endif"] + lines[738:])
    src = tmp_path / "ls9.c"
    src.write_text("\n".join(patched))
    lib = os.path.join(ROOT, "pn_gb300", "_lib")
    exe = tmp_path / "ls9_gpu"
    r = subprocess.run(["gcc", "-O2", "-w", "-DPN_GPU", "-I", os.path.join(ROOT, "include"),
                        str(src), "-L", lib, "-lpn", "-Wl,-rpath," + lib, "-lm", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    syms = subprocess.run(["nm", "-D", "--undefined-only", str(exe)], capture_output=True,
                          text=True).stdout.split()
    for s in ("force", "energy", "initial_energy"):
        assert s in syms  # resolved from libpn at run time, not defined in the binary
