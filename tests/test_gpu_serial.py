"""Tapes created from CasADi's serialized text (casadi_gb300_tape_deserialize): the rollout's
sweeps on the deserialized tape give the bits of the tape built in memory, and match the
oracle; a serialized function with calls is decoded and inlined like
casadi_gb300_tape_create_calls."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import runtime as R
from casadi_gb300 import workloads as W
from oracle import serialize as SZ

from helpers import assert_bitexact, assert_close, call_rollout_serializable, value_bounds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(arrs):
    return [None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def host(ts):
    torch.cuda.synchronize()
    return [None if t is None else t.cpu().numpy() for t in ts]


@pytest.mark.parametrize("debug,saved_form", [(False, False), (True, True)])
def test_deserialized_rollout_gives_the_in_memory_bits(gpu_lib, debug, saved_form):
    F = W.cartpole_rollout(20)
    text = SZ.serialize(SZ.from_function(F, name_in=["x0", "U"], name_out=["xN", "cost"]),
                        debug=debug, saved_form=saved_form)
    ct = R.CudaTape.deserialize(text)
    assert ct.name == F.name and ct.name_in == ["x0", "U"] and ct.name_out == ["xN", "cost"]
    assert ct.nnz_in == [4, 20] and ct.nnz_out == [4, 1]
    ref = R.CudaTape(F)
    n = 3000
    x0, U = W.cartpole_inputs(n, steps=20, seed=21)
    args = dev([x0, U])
    seeds = dev([np.zeros((1, 4, n)), np.ones((1, 1, n))])
    got = ct.jacobian_reverse(args, seeds)
    want = ref.jacobian_reverse(args, seeds)
    for g, w in zip(got, want):
        for a, b in zip(host(g), host(w)):
            assert_bitexact(a, b, "deserialized vs in-memory tape")
    vals = O.eval(F.tape, [x0, U], n)
    for a, b, vb in zip(host(got[0]), vals, value_bounds(F.tape, [x0, U], n)):
        assert_close(a, b, "values vs oracle", bound=vb)
    ct.sync()
    ref.sync()


def test_deserialized_calls_are_inlined(gpu_lib):
    steps, n = 3, 1025
    caller, step, calls = call_rollout_serializable(steps)
    ct = R.CudaTape.deserialize(SZ.serialize(caller, saved_form=True))
    step_t = R.CudaTape(step)
    inl = R.CudaTape(caller.tape, calls=[(step_t, d, r) for d, r in calls])
    x0, U = W.cartpole_inputs(n, steps=steps, seed=4)
    args = dev([x0, U])
    assert_bitexact(host(ct.eval(args))[0], host(inl.eval(args))[0], "deserialized calls")
    flat = W.cartpole_rollout(steps).tape
    want = O.eval(flat, [x0, U], n)[0]
    assert_close(host(ct.eval(args))[0], want, "calls vs oracle",
                 bound=value_bounds(flat, [x0, U], n)[0])
    ct.sync()


def test_other_classes_are_refused(gpu_lib):
    import os
    from helpers import GOLDEN
    text = open(os.path.join(GOLDEN, "serialized_issue3074.txt")).read()
    with pytest.raises(R.CasadiGpuError, match="only SXFunction"):
        R.CudaTape.deserialize(text)


def test_push_file_loads_every_function(gpu_lib, tmp_path):
    caller, step, calls = call_rollout_serializable(3)
    path = tmp_path / "functions.casadi"
    path.write_text(SZ.serialize_vector([caller.calls[0][0], caller]))
    n0 = len(R.loaded_names())
    tapes = R.push_file(str(path))
    assert R.loaded_names()[n0:] == [step.name, "rollout_calls"]
    n = 777
    x0, U = W.cartpole_inputs(n, steps=3, seed=8)
    args = dev([x0, U])
    xN = host(tapes["rollout_calls"].eval(args))[0]
    x = args[0]
    for k in range(3):
        x = tapes[step.name].eval([x, args[1][k:k + 1].contiguous()])[0]
    assert_bitexact(xN, host([x])[0], "loaded caller vs loaded step, chained")
    torch.cuda.synchronize()
    R.pop_file()
    assert len(R.loaded_names()) == n0


def test_package_load_and_deserialize(gpu_lib, tmp_path):
    import casadi_gb300 as cg
    F = W.cartpole_step()
    path = tmp_path / "step.casadi"
    path.write_text(SZ.serialize(F, saved_form=True))
    a, b = cg.load(str(path)), cg.deserialize(SZ.serialize(F))
    args = dev(W.cartpole_inputs(300, steps=1, seed=2))
    assert_bitexact(host(a.eval(args))[0], host(b.eval(args))[0], "load vs deserialize")
    a.sync()
