"""Batching form on the GPU: every register of a batch ends as the single-register engine leaves
it, alone and in the mix.

Amplitudes are compared with the plain engine (qvnt's own f64 operand order, bit-exact against the
oracle) within 1e-12 max-abs; measured values with a register-by-register QReg on the same draw.
Registers above 12 qubits run as several tiles per pass, so their passes wait on each other inside
the persistent kernel; `set_fusion(8)` makes even small registers multi-tile."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _workload(count, seed, q_range, depth_range, measure):
    from qvnt_gb300.circuits import batch_workload

    return batch_workload(count=count, seed=seed, q_range=q_range, depth_range=depth_range, measure=measure)


def _single(w, i, engine):
    from qvnt_gb300 import QReg

    q = QReg.with_state(int(w.q_nums[i]), int(w.states[i]))
    q.set_engine(engine)
    ptr, cnt = w.gates_of(i)
    q.apply_gates(ptr, cnt)
    return q


def test_batch_amplitudes_match_plain_engine():
    from qvnt_gb300 import ENGINE_PLAIN
    from qvnt_gb300.batch import Batch

    w = _workload(20, 31, (4, 15), (2, 6), measure=False)
    b = Batch(w.q_nums, w.states, w.gates, w.offsets, w.masks)
    out = b.run()
    assert np.all(out == 0)
    for i in range(w.count):
        want = _single(w, i, ENGINE_PLAIN).amplitudes()
        got = b.amplitudes(i)
        assert np.max(np.abs(got - want)) <= TOL, (i, int(w.q_nums[i]))
    # a second replay of the graph starts again from the basis states
    b.run()
    for i in (0, w.count - 1):
        want = _single(w, i, ENGINE_PLAIN).amplitudes()
        assert np.max(np.abs(b.amplitudes(i) - want)) <= TOL
    b.close()


@pytest.mark.parametrize("fusion_k,budget", [(8, 0), (10, 60), (12, 800)])
def test_batch_fusion_widths(fusion_k, budget):
    from qvnt_gb300 import ENGINE_PLAIN
    from qvnt_gb300.batch import Batch

    w = _workload(8, 41 + fusion_k, (9, 14), (3, 5), measure=False)
    b = Batch(w.q_nums, w.states, w.gates, w.offsets, w.masks)
    b.set_fusion(fusion_k, budget)
    info = b.info()
    assert info["fusion_k"] == fusion_k
    b.run()
    for i in range(w.count):
        want = _single(w, i, ENGINE_PLAIN).amplitudes()
        assert np.max(np.abs(b.amplitudes(i) - want)) <= TOL, (i, int(w.q_nums[i]))
    b.close()


def test_batch_measure_matches_registers():
    from qvnt_gb300 import ENGINE_FUSED
    from qvnt_gb300.batch import Batch
    from qvnt_gb300.circuits import SplitMix64

    w = _workload(24, 53, (4, 14), (3, 8), measure=True)
    rng = SplitMix64(77)
    u01 = np.array([rng.uniform() for _ in range(w.count)])
    b = Batch(w.q_nums, w.states, w.gates, w.offsets, w.masks)
    got = b.run(u01)
    for i in range(w.count):
        q = _single(w, i, ENGINE_FUSED)
        want = q.measure_mask(int(w.masks[i]), u01=float(u01[i]))
        assert int(got[i]) == want.get(), i
        # collapse without renormalisation: the state keeps one amplitude
        amps = b.amplitudes(i)
        assert np.count_nonzero(amps) == 1 and amps[int(got[i])] != 0
        assert np.max(np.abs(amps - q.amplitudes())) <= TOL
    b.close()


def test_batch_partial_masks_and_alone_vs_mix():
    """A register's result is the same alone and inside a larger batch."""
    from qvnt_gb300.batch import Batch
    from qvnt_gb300.circuits import batch_workload

    w = batch_workload(count=12, seed=61, q_range=(5, 13), depth_range=(2, 6), measure=True)
    w.masks = np.array([(int(m) & 0b1011) for m in w.masks], dtype=np.uint64)
    u01 = np.linspace(0.05, 0.95, w.count)
    mix = Batch(w.q_nums, w.states, w.gates, w.offsets, w.masks)
    got = mix.run(u01)
    for i in (0, 5, 11):
        a, bnd = int(w.offsets[i]), int(w.offsets[i + 1])
        alone = Batch(w.q_nums[i:i + 1], w.states[i:i + 1], w.gates_of(i)[0], np.array([0, bnd - a]),
                      w.masks[i:i + 1])
        r = alone.run(u01[i:i + 1])
        assert int(r[0]) == int(got[i])
        assert np.max(np.abs(alone.amplitudes(0) - mix.amplitudes(i))) <= TOL
        alone.close()
    mix.close()


def test_batch_autotune_and_errors():
    from qvnt_gb300._abi import QvntError
    from qvnt_gb300.batch import Batch

    w = _workload(16, 71, (8, 14), (2, 4), measure=True)
    b = Batch(w.q_nums, w.states, w.gates, w.offsets, w.masks)
    k, budget, ms = b.autotune(stride=2)
    assert k in (11, 12) and budget in (200, 400, 800, 1600) and ms > 0
    assert b.info()["fusion_k"] == k
    with pytest.raises(QvntError):
        b.run()  # measuring batches need draws
    with pytest.raises(QvntError):
        b.run(np.full(w.count, 1.0))
    b.close()
    with pytest.raises(QvntError):
        Batch([3], [0], None, [0, 0])  # below the batch's register range
    with pytest.raises(QvntError):
        Batch([5], [32], None, [0, 0])  # basis state out of range
