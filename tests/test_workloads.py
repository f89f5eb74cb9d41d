"""The seeded synthetic workloads the benchmarks run (CPU): the 4096-call
batch (m, n, k log-uniform in [16, 2048], seed 7) and the Poisson serving
stream (20,000 requests at 20k req/s, seeds 11 and 12) must stay the
workloads the recorded measurements were taken on."""
import numpy as np

from exoblas_gb300 import workloads


def test_batch_shapes_are_the_measured_batch():
    a = workloads.batch_shapes()
    assert a == workloads.batch_shapes()  # deterministic
    assert len(a) == 4096
    counts = {op: sum(1 for s in a if s[0] == op) for op in workloads.OPS}
    assert counts == {"sgemm": 1351, "dgemv": 1402, "strsv": 1343}
    dims = np.array([s[1:] for s in a])
    assert dims.min() >= 16 and dims.max() <= 2048
    # sgemm calls the batch plan sends to the tensor cores (m, n, k >= 128)
    assert sum(1 for op, m, n, k in a if op == "sgemm" and min(m, n, k) >= 128) == 232
    # log-uniform: about as many dimensions below the geometric midpoint as above
    mid = np.sqrt(16 * 2048)
    assert 0.45 < float(np.mean(dims < mid)) < 0.55


def test_serve_stream_is_the_measured_stream():
    s = workloads.serve_stream(20000)
    assert s == workloads.serve_stream(20000)
    t = np.array([r[0] for r in s])
    assert t[0] == 0.0 and np.all(np.diff(t) >= 0)
    assert abs(t[-1] - 1.0) < 0.05  # mean 20k arrivals per second
    ops = [r[1] for r in s]
    share = {op: ops.count(op) / len(ops) for op in set(ops)}
    want = {name: p for name, p in workloads.SERVE_MIX}
    total = sum(want.values())
    for op, p in want.items():
        assert abs(share.get(op, 0.0) - p / total) < 0.02, (op, share.get(op))
    prec = np.array([r[2] for r in s])
    assert abs(float(np.mean(prec == 1)) - 0.7) < 0.02
    dims = np.array([r[3:] for r in s])
    assert dims.min() >= 32 and dims.max() <= 8192
