"""Single runs of the engine's workloads, for profilers and quick checks:

    python -m qvnt_gb300.cases precision --qubits 26 --depth 8   # precision engine, random layers
    python -m qvnt_gb300.cases fused --qubits 26 --depth 8       # double-float engine, random layers
    python -m qvnt_gb300.cases batch --count 256                 # one batch run (fusion 12, budget 800)

Each builds the seeded workload, runs it once on cuda:0 and prints a one-line summary.
"""
import argparse
import time

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["precision", "fused", "batch"])
    ap.add_argument("--qubits", type=int, default=26)
    ap.add_argument("--depth", type=int, default=8)
    ap.add_argument("--count", type=int, default=256)
    ap.add_argument("--seed", type=int, default=3)
    a = ap.parse_args(argv)
    from qvnt_gb300 import ENGINE_FUSED, ENGINE_PRECISION, QReg
    from qvnt_gb300.circuits import SplitMix64, batch_workload, random_layers_gates

    t0 = time.perf_counter()
    if a.case == "batch":
        from qvnt_gb300.batch import Batch

        w = batch_workload(count=a.count, seed=4)
        b = Batch(w.q_nums, w.states, w.gates, w.offsets, w.masks)
        b.set_fusion(12, 800)
        b.run(np.full(w.count, 0.5))
        print("batch", a.count, b.info(), "%.2f s" % (time.perf_counter() - t0))
        b.close()
        return
    arr, cnt = random_layers_gates(a.qubits, a.depth, SplitMix64(a.seed))
    engine = ENGINE_PRECISION if a.case == "precision" else ENGINE_FUSED
    q = QReg(a.qubits, 0, engine=engine)
    q.apply_gates(arr, cnt)
    q.sync()
    launches, passes = q.stats()
    print(a.case, a.qubits, "gates", cnt, "passes", passes, "%.2f s" % (time.perf_counter() - t0))
    q.close()


if __name__ == "__main__":
    main()
