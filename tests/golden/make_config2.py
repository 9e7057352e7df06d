"""Writes tests/golden/config2_26q.npz: the oracle's result for the config-2 generator (random
layers of {h, s, t, u3}, 15 two-qubit gates and 3 Toffolis per layer, depth 40, then op::qft over
all qubits) at 26 qubits, seed 2 (2,633 gates): a register the oracle finishes in a few minutes on 8 cores.

    python tests/golden/make_config2.py [--qubits 26] [--depth 40] [--seed 2]

The circuit is built with the oracle's own builders (oracle_ref.random_circuit_gates) and applied
with the oracle (one out-of-place pass per gate, qvnt's MultiOp::apply).  Stored:
  gates_sha256   hash of the gate list bytes (the engine's generator must give the same list)
  norm           get_absolute (sum of |psi|^2) of the whole register
  idx, amp       4,096 amplitudes at seeded indices plus the first 64
  chunk_norms    sum of |psi|^2 over each of 256 equal contiguous chunks
  psi_sum        sum of all amplitudes (complex)
  draws, chosen  WeightedIndex choices (measure_mask of every qubit) for fixed uniform draws
Test infrastructure only: run here, committed as a fixture.
"""
import argparse
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle_ref as orc  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--qubits", type=int, default=26)
    ap.add_argument("--depth", type=int, default=40)
    ap.add_argument("--seed", type=int, default=2)
    a = ap.parse_args()
    n = a.qubits
    gates = orc.random_circuit_gates(n, a.depth, seed=a.seed)
    sha = hashlib.sha256(b"".join(bytes(g) for g in gates)).hexdigest()
    psi = orc.new_state(n, 0)
    t0 = time.time()
    orc.apply(gates, psi)
    dt = time.time() - t0
    rng = orc.SplitMix64(99)
    idx = np.array(sorted(set([rng.below(1 << n) for _ in range(4096)]) | set(range(64))), dtype=np.uint64)
    probs = orc.get_probabilities(psi, n)
    draws = np.array([0.0, 1e-9, 0.1, 0.25, 0.37, 0.5, 0.73, 0.9, 0.999999], dtype=np.float64)
    chosen = np.array([orc.weighted_index(probs, u) for u in draws], dtype=np.uint64)
    chunks = np.abs(psi[: 1 << n].reshape(256, -1)) ** 2
    np.savez_compressed(os.path.join(HERE, "config2_%dq.npz" % n), qubits=n, depth=a.depth, seed=a.seed,
                        gate_count=len(gates), gates_sha256=sha, norm=orc.get_absolute(psi), idx=idx,
                        amp=psi[idx.astype(np.int64)], chunk_norms=chunks.sum(axis=1), psi_sum=psi.sum(),
                        draws=draws, chosen=chosen)
    print("config2 %dq: %d gates, oracle %.1f s, norm %.17g" % (n, len(gates), dt, orc.get_absolute(psi)))


if __name__ == "__main__":
    main()
