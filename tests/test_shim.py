"""The QLens-side shim (oracle/qlpix_shim.cpp, the code INTEGRATION.md
describes) compiles against the unmodified reference's headers and objects,
links with libqlpix, and -- without a GPU -- qlp_create refuses cleanly with
QLP_ERR_NO_DEVICE (there is no CPU fallback).  With a GPU the same program
evaluates the golden case through the shim and compares -2 log(evidence) with
the reference's own entry point.  Needs the reference build (oracle/_ref,
made by build() where the reference sources are present); skipped elsewhere."""
import os
import subprocess

import pytest

from goldens import Golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "oracle", "_ref", "qlpix_shim_check")


@pytest.mark.skipif(not os.path.exists(SHIM), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("case", ["tiny_sie", "powerlaw"])
def test_shim_builds_links_and_refuses_without_a_gpu(case, tmp_path):
    import torch
    script = tmp_path / "case.in"
    script.write_text(Golden(case).meta["script"])
    r = subprocess.run([SHIM, str(script)], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-1000:] + r.stderr[-1000:]
    if torch.cuda.is_available():
        assert "qlpix -2logev" in r.stdout
    else:
        assert "no device: qlp_create refused" in r.stdout
