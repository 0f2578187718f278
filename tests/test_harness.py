"""The C++ harness (bitwise_spgemm_gb300/harness/bsp_harness): the reference
main()'s pipeline — pack, group, plan, SpMM, exact check — through the C
ABI alone."""
import os
import subprocess

import pytest

from bitwise_spgemm_gb300 import build as B

HARNESS = B.HARNESS


def _built():
    if not os.path.exists(HARNESS):
        B.build()
    return HARNESS


def test_harness_links_and_rejects_bad_sizes():
    # runs without a GPU: size checks come before any CUDA call
    r = subprocess.run([_built(), "0", "16", "16"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 2 and "bad sizes" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("args,env", [(["2048", "2048", "256", "0.05", "1"], {}),
                                      (["1000", "3000", "96", "0.1", "2", "--bf16"], {"BSP_TC": "1"}),
                                      (["4096", "1024", "512", "0.3", "3", "--bf16"], {"BSP_TC": "0"}),
                                      (["300", "70", "8", "0.5", "4"], {})])
def test_harness_pipeline_passes(args, env):
    r = subprocess.run([_built()] + args, capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, **env))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "check=PASS" in r.stdout and "mismatches=0" in r.stdout
