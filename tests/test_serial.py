"""Decoding CasADi's serialized Functions on the host (casadi_gb300_serialized_describe /
_decode; the GPU entry casadi_gb300_tape_deserialize is in test_gpu_serial.py).

The common layers (stream header and primitives, shared objects, the ProtoFunction and
FunctionInternal bodies in their old versions, Sparsity, the saved form) are checked against
the one serialized Function the reference's tests hold (tests/golden/serialized_issue3074.txt,
an MXFunction). The SXFunction layers are checked by round trips through the writer restated
in oracle/serialize.py, in plain and debug mode and in both top-level forms."""
import os

import numpy as np
import pytest

from casadi_gb300 import runtime as R
from casadi_gb300 import workloads as W
from oracle import serialize as SZ

from helpers import GOLDEN, call_rollout_serializable


@pytest.fixture(scope="module")
def lib():
    try:
        return R.load()
    except Exception as e:  # the library is built by __graft_entry__.build()
        pytest.skip("library not built: %s" % e)


def reference_text():
    with open(os.path.join(GOLDEN, "serialized_issue3074.txt")) as fh:
        return fh.read()


def test_reference_blob_common_layers(lib):
    d = R.describe_serialized(reference_text())
    assert d["saved_form"] and not d["debug"] and d["top"] == 0
    (f,) = d["functions"]
    assert f["class"] == "MXFunction" and f["name"] == "delay_arguments"
    # ProtoFunction v1, FunctionInternal v2 (an earlier CasADi), then the XFunction header:
    # its input count equals the FunctionInternal's, so every field before it was read with
    # its right width
    assert f["versions"][:3] == [1, 2, 1] and not f["complete"]
    assert f["x_inputs"] == len(f["inputs"]) == 7
    assert [i["name"] for i in f["inputs"]] == ["i%d" % k for k in range(7)]
    assert [i["size"] for i in f["inputs"]] == [[1, 1], [2, 1], [2, 1], [6, 1], [0, 1], [0, 1],
                                                [4, 1]]
    assert [i["nnz"] for i in f["inputs"]] == [1, 2, 2, 6, 0, 0, 4]
    assert f["outputs"] == []
    # the same text from a file path
    assert R.describe_serialized(os.path.join(GOLDEN, "serialized_issue3074.txt")) == d
    # not an SXFunction: no tape
    with pytest.raises(R.CasadiGpuError, match="MXFunction"):
        R.decode_serialized(reference_text())


FUNCTIONS = {
    "cartpole_step": lambda: W.cartpole_step(),
    "rollout20": lambda: W.cartpole_rollout(20),
    "dag": lambda: W.random_dag(n_in=16, n_nodes=800, n_out=6, seed=3),
}


@pytest.mark.parametrize("name", sorted(FUNCTIONS))
@pytest.mark.parametrize("debug", [False, True])
@pytest.mark.parametrize("saved_form", [False, True])
def test_sx_round_trip(lib, name, debug, saved_form):
    F = FUNCTIONS[name]()
    text = SZ.serialize(SZ.from_function(F, name_in=["a%d" % j for j in range(F.n_in())]),
                        debug=debug, saved_form=saved_form)
    t = R.decode_serialized(text)
    want, got = SZ.tape_arrays(F.tape), SZ.tape_arrays(t)
    for a, b in zip(want[:3], got[:3]):
        assert np.array_equal(a, b)  # op, i0 and the 8-byte payload (constants bit for bit)
    assert want[3:] == got[3:]
    d = R.describe_serialized(text)
    assert d["debug"] == debug and d["saved_form"] == saved_form
    f = d["functions"][d["top"]]
    assert f["class"] == "SXFunction" and f["name"] == F.name and f["complete"]
    assert f["versions"] == [2, 8, 1, 3]
    assert [i["name"] for i in f["inputs"]] == ["a%d" % j for j in range(F.n_in())]
    assert [i["nnz"] for i in f["inputs"]] == list(F.tape.nnz_in)
    assert [o["nnz"] for o in f["outputs"]] == list(F.tape.nnz_out)
    assert f["n_instr"] == F.tape.n_instr and f["sz_w"] == F.tape.sz_w
    assert f["x_inputs"] == F.n_in() and f["calls"] == [] and f["n_free"] == 0


@pytest.mark.parametrize("debug", [False, True])
def test_called_functions_are_decoded_first(lib, debug):
    caller, step, calls = call_rollout_serializable(3)
    text = SZ.serialize(caller, debug=debug, saved_form=True)
    d = R.describe_serialized(text)
    assert [f["name"] for f in d["functions"]] == [step.name, "rollout_calls"]
    assert d["top"] == 1 and d["functions"][1]["calls"] == [0, 0, 0]
    assert d["functions"][0]["n_instr"] == step.tape.n_instr
    with pytest.raises(R.CasadiGpuError, match="calls 3 functions"):
        R.decode_serialized(text)


def test_free_variables_are_refused(lib):
    from casadi_gb300 import sx as S
    F = W.cartpole_step()
    s = SZ.from_function(F, free_vars=[S.sym("p")])
    text = SZ.serialize(s)
    assert R.describe_serialized(text)["functions"][0]["n_free"] == 1
    with pytest.raises(R.CasadiGpuError, match="free variables"):
        R.decode_serialized(text)


def test_malformed_text_is_an_error(lib):
    text = SZ.serialize(W.cartpole_step())
    bad = [
        text[:-1],                         # odd length
        "q" + text[1:],                    # character outside a..p
        "",                                # nothing
        text[:40],                         # header only
        "b" + text[1:],                    # sanity check value
        text[:16] + "ea" + text[18:],      # protocol version 4 instead of 3
    ]
    # truncations all along the stream
    bad += [text[:k] for k in range(34, len(text) - 2, 997)]
    for t in bad:
        with pytest.raises(R.CasadiGpuError):
            R.describe_serialized(t)
    # trailing whitespace is ignored
    assert R.describe_serialized(text + "\n")["functions"][0]["n_instr"] == 158


def test_corrupted_bytes_never_crash(lib):
    """Byte flips all over a serialized step function: each decode either fails with an
    error status or returns a model; none reads out of bounds or allocates without bound."""
    text = SZ.serialize(W.cartpole_step(), debug=True)
    rng = np.random.default_rng(0)
    outcomes = {"error": 0, "decoded": 0}
    for _ in range(300):
        chars = list(text)
        for p in rng.integers(0, len(chars), size=int(rng.integers(1, 4))):
            chars[p] = chr(97 + int(rng.integers(0, 16)))
        try:
            R.describe_serialized("".join(chars))
            outcomes["decoded"] += 1
        except R.CasadiGpuError:
            outcomes["error"] += 1
    assert outcomes["error"] > 0 and sum(outcomes.values()) == 300


@pytest.mark.parametrize("debug", [False, True])
def test_function_vector_files(lib, debug, tmp_path):
    """The FileSerializer form of a vector of Functions (type byte 15), as casadi_c_push_file
    reads it: every Function is listed as a top-level one, called ones once."""
    caller, step, _ = call_rollout_serializable(2)
    dag = W.random_dag(n_in=8, n_nodes=200, n_out=3, seed=1)
    text = SZ.serialize_vector([caller.calls[0][0], caller, dag], debug=debug)
    d = R.describe_serialized(text)
    names = [d["functions"][k]["name"] for k in d["tops"]]
    assert names == [step.name, "rollout_calls", dag.name] and d["top"] == -1
    assert len(d["functions"]) == 3  # the step function is written once, then referenced
    with pytest.raises(R.CasadiGpuError, match="holds 3 Functions"):
        R.decode_serialized(text)


def test_push_file_refuses_other_classes(lib, tmp_path):
    n0 = len(R.loaded_names())
    with pytest.raises(R.CasadiGpuError, match="MXFunction"):
        R.push_file(os.path.join(GOLDEN, "serialized_issue3074.txt"))
    with pytest.raises(R.CasadiGpuError, match="could not open"):
        R.push_file(str(tmp_path / "missing.casadi"))
    p = tmp_path / "plain.txt"
    p.write_text(SZ.serialize(W.cartpole_step()))  # Function::serialize() text, not a file
    with pytest.raises(R.CasadiGpuError, match="no 'function'"):
        R.push_file(str(p))
    assert len(R.loaded_names()) == n0


def test_deep_nesting_is_an_error_not_a_crash(lib):
    """Option dictionaries nest by recursion in the reader: 300 levels are refused, 50 read."""
    def nested(depth):
        d = {"leaf": 1.5}
        for k in range(depth):
            d = {"level%d" % k: d}
        return d
    import sys
    F = W.cartpole_step()
    limit = sys.getrecursionlimit()
    sys.setrecursionlimit(max(limit, 10000))  # the writer recurses into nested values too
    try:
        ok = SZ.serialize(SZ.from_function(F, jit_options=nested(50)))
        deep = SZ.serialize(SZ.from_function(F, jit_options=nested(300)))
    finally:
        sys.setrecursionlimit(limit)
    assert R.decode_serialized(ok).n_instr == F.tape.n_instr
    with pytest.raises(R.CasadiGpuError, match="nested deeper"):
        R.describe_serialized(deep)


@pytest.mark.parametrize("debug", [False, True])
def test_empty_io_and_constant_kinds(lib, debug):
    """An empty input and an empty output (0x1 patterns, as in the reference's blob) and
    constants of every ConstantSX kind the writer emits (0, 1, -1, integers, reals, inf, nan):
    the tape's constants come back bit for bit from the algorithm's i1/i2 words."""
    from casadi_gb300 import sx as S
    x = S.sym("x", 2)
    outs = [[x[0] * 2.5 + 1.0, x[1] - 1.0, x[0] * 0.0 + 3.0, x[1] * float("inf"),
             x[0] + (-7.0), x[1] * float("nan"), x[0] * -1.0 + 0.1], []]
    F = S.Function("edge", [[], x], outs)
    text = SZ.serialize(F, debug=debug)
    t = R.decode_serialized(text)
    want, got = SZ.tape_arrays(F.tape), SZ.tape_arrays(t)
    for a, b in zip(want[:3], got[:3]):
        assert np.array_equal(a, b)
    assert got[3] == [0, 2] and got[4] == [7, 0]
    f = R.describe_serialized(text)["functions"][0]
    assert [i["size"] for i in f["inputs"]] == [[0, 1], [2, 1]]
    assert [o["nnz"] for o in f["outputs"]] == [7, 0]
