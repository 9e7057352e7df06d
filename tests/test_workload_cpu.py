"""The synthetic workload generators: the library's C twin (qvnt_workload_random_layers) draws the
same gates as the Python generator, and the batching workload has the configured shape."""
import numpy as np
import pytest

pytestmark = pytest.mark.usefixtures("lib_built")


@pytest.mark.parametrize("n,depth,seed", [(3, 2, 1), (5, 3, 7), (9, 4, 11), (20, 2, 5)])
def test_c_generator_matches_python(n, depth, seed):
    from qvnt_gb300.circuits import SplitMix64, _concat, random_layers, random_layers_gates

    r1 = SplitMix64(seed)
    gates = _concat(random_layers(n, depth, r1)).gates()
    r2 = SplitMix64(seed)
    arr, count = random_layers_gates(n, depth, r2)
    assert count == len(gates)
    for i in range(count):
        assert bytes(arr[i]) == bytes(gates[i]), i
    assert r1.state == r2.state


def test_batch_workload_shape():
    from qvnt_gb300.circuits import batch_workload

    w = batch_workload(count=64, seed=9, q_range=(8, 20), depth_range=(10, 60))
    assert w.count == 64
    assert w.q_nums.min() >= 8 and w.q_nums.max() <= 20
    assert w.depths.min() >= 10 and w.depths.max() <= 60
    assert all(int(s) < (1 << int(n)) for s, n in zip(w.states, w.q_nums))
    assert np.all(np.diff(w.offsets.astype(np.int64)) > 0)
    assert all(int(m) == (1 << int(n)) - 1 for m, n in zip(w.masks, w.q_nums))
    # every gate of register i acts inside register i
    from qvnt_gb300._abi import lib

    for i in range(w.count):
        ptr, cnt = w.gates_of(i)
        lim = 1 << int(w.q_nums[i])
        for j in range(cnt):
            g = ptr[j]
            assert (lib().qvnt_gate_act_on(ptr[j]) | g.ctrl) < lim


@pytest.mark.parametrize("n", [12, 13, 16, 24, 32])
def test_precision_planner_terminates(n):
    """The precision engine's host planner places every dense block (it fuses the config-3 layers
    at about ten gates per block)."""
    import ctypes

    from qvnt_gb300._abi import check, lib
    from qvnt_gb300.circuits import SplitMix64, random_layers_gates

    arr, cnt = random_layers_gates(n, 12, SplitMix64(n))
    p, b = ctypes.c_uint64(), ctypes.c_uint64()
    check(lib().qvnt_precision_plan_info(arr, cnt, n, ctypes.byref(p), ctypes.byref(b)))
    assert 0 < b.value <= cnt and 0 < p.value <= b.value


@pytest.mark.parametrize("n,depth,seed", [(5, 3, 2), (24, 40, 2), (30, 40, 2)])
def test_oracle_builders_give_the_same_circuit(n, depth, seed):
    """The oracle-built workload (the CPU baseline's and the reference arm's circuit) is the
    library-built one byte for byte, the config-2 shape included."""
    import oracle_ref as orc
    from qvnt_gb300.circuits import plain_circuit, random_circuit

    a = [bytes(g) for g in random_circuit(n, depth, seed=seed).gates()]
    b = [bytes(g) for g in orc.random_circuit_gates(n, depth, seed=seed)]
    assert a == b
    if n == 5:
        a = [bytes(g) for g in plain_circuit(20, 20, seed=1).gates()]
        assert a == [bytes(g) for g in orc.plain_circuit_gates(20, 20, seed=1)]
