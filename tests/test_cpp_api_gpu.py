"""The C++ drop-in header (include/bem_gb300.hpp): a C++ program running the
reference driver's call sequence (main.cpp) through it reproduces the
reference's golden output and the oracle's answer for the same steps."""
import os
import subprocess

import numpy as np
import pytest

from helpers import FIELD_GOLDEN, GOLDEN, K_GOLDEN, chief_candidates, float_bb, golden, read_cplx_file

pytestmark = pytest.mark.gpu


def test_cpp_driver_golden(bemlib, orc, tmp_path):
    from bem_gpu_clean_cpp_gb300 import build
    exe = build.DRIVER
    assert os.path.exists(exe)
    out = tmp_path / "sphere171Hz_CHIEF"
    res = subprocess.run([exe, f"{GOLDEN}/sphere.obj", str(out), "171.5", "1", "0.1"],
                         capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    got = read_cplx_file(str(out))
    g = golden("sphere171Hz_CHIEF")
    assert got.shape == g.shape
    assert (np.abs(got - g) / np.abs(g)).max() < 5e-3
    # the oracle running the same steps in FP64
    p, f = orc.read_obj_reference(f"{GOLDEN}/sphere.obj")
    p = p.astype(np.float64)
    ch, _ = orc.chief_select(p, f, float_bb(p, 1e-4), 0.1, chief_candidates(), 1)
    src = [("point", (1e6, 1e6, 1e6), 0.0)]
    A, B = orc.assemble(np.vstack([p, ch.astype(np.float32).astype(np.float64)]), f, K_GOLDEN, p.shape[0], src)
    x = orc.lsq_qr(A, B)[:, 0]
    ref = np.concatenate([[x[0]], orc.field(p, f, K_GOLDEN, x, FIELD_GOLDEN, src)[:, 0]])
    assert (np.abs(got - ref) / np.abs(ref)).max() < 2e-4
