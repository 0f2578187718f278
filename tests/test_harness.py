"""The C++ harness (bitwise_spgemm_gb300/harness/bsp_harness): the reference
main()'s pipeline — pack, group, plan, SpMM, exact check — through the C
ABI alone."""
import os
import subprocess

import pytest

from bitwise_spgemm_gb300 import build as B

HARNESS = B.HARNESS
E2E = B.E2E


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


def test_e2e_driver_rejects_bad_arguments():
    exe = E2E if os.path.exists(E2E) else B.build_e2e()
    r = subprocess.run([exe, "/nonexistent", "0", "16", "16", "1", "0", "0"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 2 and "bad sizes" in r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("reuse", ["0", "1", "2"])
def test_e2e_driver_serving_loop(tmp_path, reuse):
    """The C++ serving loop (uploads, plan, SpMM, download, two steps in
    flight) through the C ABI: its last C equals the oracle's exact sum for
    integer-valued B, with the plan built every step and reused."""
    import json
    import numpy as np
    import oracle as O
    from bitwise_spgemm_gb300 import workloads as W
    exe = E2E if os.path.exists(E2E) else B.build_e2e()
    A, _, _ = W.clustered_bits(1024, 2048, n_proto=8, p_proto=0.05, p_flip=0.003, seed_proto=5, seed_rows=6)
    words = W.pack_bits(A)
    Bi = np.random.default_rng(7).integers(-8, 9, (2048, 256)).astype(np.float32)
    words.tofile(str(tmp_path / "words.bin"))
    Bi.tofile(str(tmp_path / "B.bin"))
    r = subprocess.run([exe, str(tmp_path), "1024", "2048", "256", "5", "2", reuse], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["device_status"] == 0 and line["ms_per_step"] > 0
    if reuse == "2":  # copies alone: no product
        assert line["plan"].startswith("none")
        return
    C = np.fromfile(str(tmp_path / "C.bin"), np.float32).reshape(1024, 256)
    assert np.array_equal(C.astype(np.float64), O.spmm_f64(words, 2048, Bi))
