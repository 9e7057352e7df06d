"""The allocation-free norm entry point, qvnt_norm_sqr_noalloc, for callers that cannot call
cudaMalloc (their device memory belongs to their own allocator or pool, or an allocation would
synchronise the device mid-stream).

The caller owns both device buffers (here torch tensors stand in for the caller's memory); the
entry point itself allocates nothing and keeps its partial sums in a file-scope device array.  Its
result must equal the register API's qvnt_reg_get_absolute on the same state, on two calls in a
row (the second call reuses the array the first one left behind).  This file is collected last so
that a failure here comes after every other test has run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _sum_noalloc(lib, d_psi, n_amps, d_out, stream):
    st = lib.qvnt_norm_sqr_noalloc(ctypes.c_void_p(d_psi), n_amps, ctypes.c_void_p(d_out), ctypes.c_void_p(stream))
    assert st == 0, lib.qvnt_last_error().decode()


def test_norm_noalloc_matches_register_api():
    torch = pytest.importorskip("torch")
    from qvnt_gb300 import ENGINE_PLAIN, QReg, _abi
    from qvnt_gb300.circuits import random_circuit

    lib = _abi.lib()
    for n in (14, 21):
        q = QReg.new(n)
        q.set_engine(ENGINE_PLAIN)
        q.apply(random_circuit(n, 4, seed=5 + n))
        q.measure_mask(0b11, 0.3)  # collapse without renormalising: the norm is no longer 1
        want = q.get_absolute()
        psi = q.amplitudes()
        dev = torch.device("cuda", 0)
        d_psi = torch.from_numpy(psi.view(np.float64).copy()).to(dev)
        d_out = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        results = []
        for _ in range(2):  # two calls in a row: the second reuses the scratch the first left behind
            d_out.fill_(-1.0)
            _sum_noalloc(lib, d_psi.data_ptr(), psi.size, d_out.data_ptr(), stream)
            torch.cuda.synchronize(dev)
            results.append(float(d_out.item()))
        for got in results:
            assert abs(got - want) <= TOL, (n, got, want)
        assert 0.0 < want < 1.0


def test_norm_noalloc_ragged_lengths():
    """Lengths that are not multiples of the 4096-amplitude chunk (a single partial chunk, a ragged
    last chunk) against numpy's sum of |psi|^2, twice in a row."""
    torch = pytest.importorskip("torch")
    from qvnt_gb300 import _abi

    lib = _abi.lib()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(8)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for n_amps in (8, 17, 4095, 5000, 4096 * 3 + 17, 4096 * 37 + 1):
        host = rng.normal(size=2 * n_amps)
        want = float(np.sum(host * host))
        d_psi = torch.from_numpy(host.copy()).to(dev)
        d_out = torch.empty(1, dtype=torch.float64, device=dev)
        for _ in range(2):
            d_out.fill_(-1.0)
            _sum_noalloc(lib, d_psi.data_ptr(), n_amps, d_out.data_ptr(), stream)
            torch.cuda.synchronize(dev)
            got = float(d_out.item())
            assert abs(got - want) <= 1e-12 * want, (n_amps, got, want)


def test_norm_noalloc_rejects_oversized_state():
    from qvnt_gb300 import _abi

    lib = _abi.lib()
    st = lib.qvnt_norm_sqr_noalloc(ctypes.c_void_p(16), (1 << 28) + 1, ctypes.c_void_p(16), None)
    assert st == _abi.ERR_BAD_ARG
    assert b"allocation-free limit" in lib.qvnt_last_error()
