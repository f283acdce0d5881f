"""The CudaMap plugin (casadi_gb300/plugin) compiled against the reference's own libcasadi
and driven through CasADi's C++ API (tests/plugin/cuda_map_check.cpp): CudaMap::create(f, 8)
of the cart-pole step is a Map of class CudaMap with the same I/O and sparsity as
f.map(8, "serial"); its numeric call matches the serial Map where a GPU is present and fails
cleanly -- the library's message as a CasADi warning, an evaluation-failed error, nothing
crossing the C ABI -- where none is. A Function::serialize() / Function::deserialize() round
trip gives a CudaMap back that behaves the same. Runs where libcasadi was built (oracle/Makefile casadi);
skipped elsewhere."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
BUILT = os.path.exists(os.path.join(ORACLE, "_ref", "libcasadi.so")) and os.path.exists(
    os.path.join(ORACLE, "_ref", "gen", "reference_tree.txt"))


@pytest.mark.skipif(not BUILT, reason="libcasadi not built here")
def test_cuda_map_plugin_through_casadis_api():
    from casadi_gb300 import build as B
    B.build()
    subprocess.check_call(["make", "-s", "-C", ORACLE, "plugin-check"])
    r = subprocess.run([os.path.join(ORACLE, "_ref", "cuda_map_check")], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    kv = dict(line.split("=", 1) for line in r.stdout.splitlines() if "=" in line)
    assert kv["class"] == "CudaMap" and kv["is_map"] == "1" and kv["is_cuda_map"] == "1"
    assert (kv["n_in"], kv["n_out"]) == ("2", "1")
    assert kv["size_in0"] == "4x8" and kv["size_out0"] == "4x8" and kv["same_sparsity"] == "1"
    for key in ("eval", "back_eval"):
        if kv[key + "_ok"] == "1":
            assert float(kv[key + "_max_abs_diff"]) <= 1e-12
        else:
            assert "Evaluation failed" in kv[key + "_error"]
            assert "CudaMap:" in r.stdout + r.stderr  # the library's message, as a warning
    # Function::deserialize of the serialized text (with Map::deserialize's "CudaMap" branch)
    # gives a CudaMap with the same I/O back
    assert kv["back_class"] == "CudaMap" and kv["back_same_sparsity"] == "1"
