"""Batched persistent execution: every instance of a mixed batch must match
the CPU oracle for the same call (1% rule and componentwise FP bound; strsv by
the residual bound), alone and inside the batch, for plain runs and
CUDA-graph replays, including the full 4096-instance batch (m, n, k
log-uniform in [16, 2048], seed 7)."""
import numpy as np
import pytest

from common import (EPS, LO, NT, NU, ROW, TR, UN, UP, Case, assert_bound, assert_rel1pct, fp64_reference, run_oracle,
                    trsv_residual_ok)


def _mixed_cases(seed=3, count=60):
    g = np.random.default_rng(seed)
    cases = []
    for i in range(count):
        kind = i % 3
        m, n, k = (int(v) for v in np.exp(g.uniform(0, np.log(300), 3)).astype(int).clip(1, 300))
        if kind == 0:
            ta, tb = (NT, TR)[i % 2], (NT, TR)[(i // 2) % 2]
            ar, ac = (m, k) if ta == NT else (k, m)
            br, bc = (k, n) if tb == NT else (n, k)
            A = g.uniform(-1, 1, ar * ac).astype(np.float32)
            B = g.uniform(-1, 1, br * bc).astype(np.float32)
            Cm = g.uniform(-1, 1, m * n).astype(np.float32)
            cases.append(Case("sgemm", [ROW, ta, tb, m, n, k, 1.5, A, ac, B, bc, 0.5, Cm, n], [12], nred=k + 1))
        elif kind == 1:
            t = (NT, TR)[i % 2]
            incx, incy = (1, 2, -1)[i % 3], (1, -2)[i % 2]
            xl, yl = (n, m) if t == NT else (m, n)
            A = g.uniform(-1, 1, m * n)
            x = g.uniform(-1, 1, 1 + (xl - 1) * abs(incx))
            y = g.uniform(-1, 1, 1 + (yl - 1) * abs(incy))
            cases.append(Case("dgemv", [ROW, t, m, n, 0.75, A, n, x, incx, 0.5, y, incy], [10], nred=xl + 1))
        else:
            u, t, d = (UP, LO)[i % 2], (NT, TR)[(i // 2) % 2], (NU, UN)[(i // 4) % 2]
            A = g.uniform(-1, 1, (m, m)) / m
            A[np.arange(m), np.arange(m)] = 1 + g.uniform(0, 1, m)
            x = g.uniform(-1, 1, m)
            cases.append(Case("strsv", [ROW, u, t, d, m, A.astype(np.float32).ravel(), m, x.astype(np.float32), 1],
                              [7], nred=m + 1))
    return cases


def _to_ops(torch, cases):
    from exoblas_gb300.batch import BatchOp

    ops, dev = [], []
    for c in cases:
        a = [torch.from_numpy(v.copy()).cuda() if isinstance(v, np.ndarray) else v for v in c.args]
        dev.append(a)
        if c.op == "sgemm":
            _, ta, tb, m, n, k, al, A, lda, B, ldb, be, Cm, ldc = a
            ops.append(BatchOp.sgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, Cm, ldc))
        elif c.op == "dgemv":
            _, t, m, n, al, A, lda, x, ix, be, y, iy = a
            ops.append(BatchOp.dgemv(t, m, n, al, A, lda, x, ix, be, y, iy))
        else:
            _, u, t, d, n, A, lda, x, ix = a
            ops.append(BatchOp.strsv(u, t, d, n, A, lda, x, ix))
    return ops, dev


def _check(case, got):
    o_r, o_a = run_oracle(case)
    j = case.outputs[0]
    assert_rel1pct(got, o_a[j], f"batch {case.op}")
    if case.op == "strsv":
        trsv_residual_ok(case, got)
        return
    (r64, a64), (m, am) = fp64_reference(case)
    assert_bound(got, a64[j], am[j], case.nred, case.p, 4.0, f"batch {case.op}")


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [False, True])
def test_mixed_batch_matches_oracle(cuda, graph):
    from exoblas_gb300.batch import BatchPlan

    torch = cuda
    cases = _mixed_cases()
    ops, dev = _to_ops(torch, cases)
    plan = BatchPlan(ops)
    assert plan.info()["units"] >= len(cases)
    if graph:
        plan.graph_launch()
    else:
        plan.run()
    torch.cuda.synchronize()
    for c, a in zip(cases, dev):
        _check(c, a[c.outputs[0]].cpu().numpy())
    plan.close()


@pytest.mark.gpu
def test_batch_result_same_alone_and_in_mix(cuda):
    """Each instance alone (a one-op plan) equals its value inside the mix."""
    from exoblas_gb300.batch import BatchPlan

    torch = cuda
    cases = _mixed_cases(seed=9, count=24)
    ops, dev = _to_ops(torch, cases)
    mixed = BatchPlan(ops)
    mixed.run()
    torch.cuda.synchronize()
    outs = [a[c.outputs[0]].cpu().numpy().copy() for c, a in zip(cases, dev)]
    ops2, dev2 = _to_ops(torch, cases)
    for i, (c, op) in enumerate(zip(cases, ops2)):
        p = BatchPlan([op])
        p.run()
        torch.cuda.synchronize()
        alone = dev2[i][c.outputs[0]].cpu().numpy()
        assert alone.tobytes() == outs[i].tobytes(), f"instance {i} ({c.op}) differs alone vs in the mix"
        p.close()


@pytest.mark.gpu
def test_autotuner_picks_valid_configs(cuda, tmp_path, monkeypatch):
    import exoblas_gb300.batch as bt

    monkeypatch.setenv("EXOBLAS_TUNE_CACHE", str(tmp_path / "tune.json"))
    for m, n, k in [(16, 16, 16), (300, 200, 100), (2048, 2048, 2048)]:
        assert bt.tile_config(m, n, k) in (0, 1, 2)


@pytest.mark.gpu
def test_full_batch_every_instance(cuda):
    """The 4096-instance batch of the benchmark (sgemm NN / dgemv N / strsv
    lower no-trans non-unit, m, n, k log-uniform in [16, 2048], seed 7) run as
    one plan: every sgemm against an FP64 product on the device within
    4 (k + 1) eps_s |A||B| + ..., every dgemv against the oracle's
    double-word gemv within 4 (n + 1) eps_d |A||x| + ..., every strsv by the
    residual bound 8 n eps_s |L||x|.  The CUDA-graph replay of the same plan
    from the same inputs must then give every output bit for bit."""
    import oracle
    from exoblas_gb300 import workloads
    from exoblas_gb300.batch import BatchPlan

    torch = cuda
    ops, shapes, arena, views = workloads.batch_config(torch, "cuda")
    assert len(views) == 4096
    outs = [t[-1] for (_, _, t) in views]  # C, y, x: updated in place
    start = [o.clone() for o in outs]
    torch.cuda.synchronize()
    plan = BatchPlan(ops)
    plan.run()
    torch.cuda.synchronize()
    ran = [o.clone() for o in outs]
    counts = {"sgemm": 0, "dgemv": 0, "strsv": 0}
    for i, ((op, dims, t), c0) in enumerate(zip(views, start)):
        counts[op] += 1
        if op == "sgemm":
            m, n, k = dims
            A, B = t[0].view(m, k).double(), t[1].view(k, n).double()
            C0 = c0.view(m, n).double()
            ref = A @ B + 0.5 * C0
            mag = A.abs() @ B.abs() + 0.5 * C0.abs()
            err = (t[2].view(m, n).double() - ref).abs()
            tol = 4.0 * (k + 1) * EPS["s"] * mag
            assert bool((err <= tol).all()), f"sgemm instance {i} {dims}: max err/tol {float((err / tol).max())}"
        elif op == "dgemv":
            m, n = dims
            A, x = t[0].cpu().numpy(), t[1].cpu().numpy()
            y0 = c0.cpu().numpy()
            _, hp = oracle.call_dw("dgemv", ROW, NT, m, n, 1.0, A, n, x, 1, 0.5, y0, 1)
            mag = np.abs(A.reshape(m, n)) @ np.abs(x) + 0.5 * np.abs(y0)
            assert_bound(t[2].cpu().numpy(), hp[10], mag, n + 1, "d", 4.0, f"dgemv instance {i} {dims}")
        else:
            (n,) = dims
            case = Case("strsv", [ROW, LO, NT, NU, n, t[0].cpu().numpy(), n, c0.cpu().numpy(), 1], [7], nred=n + 1)
            trsv_residual_ok(case, t[1].cpu().numpy())
    assert min(counts.values()) > 1200, counts
    for o, s0 in zip(outs, start):
        o.copy_(s0)
    torch.cuda.synchronize()
    plan.graph_launch()
    torch.cuda.synchronize()
    for i, (o, r) in enumerate(zip(outs, ran)):
        assert torch.equal(o, r), f"instance {i}: graph replay differs from the plan run"
    plan.close()


def _tc_cases(seed=21):
    """sgemm calls of which most reach the tensor-core group (m, n, k >= 128),
    all four transpose pairs, ragged sizes (not multiples of 128 or 64)."""
    g = np.random.default_rng(seed)
    cases = []
    for i, (m, n, k) in enumerate([(128, 128, 128), (300, 200, 130), (129, 640, 257), (1000, 130, 700),
                                   (96, 512, 512), (256, 256, 31), (517, 389, 1021), (63, 1999, 128),
                                   (64, 64, 32), (70, 1030, 40)]):
        ta, tb = (NT, TR)[i % 2], (NT, TR)[(i // 2) % 2]
        ar, ac = (m, k) if ta == NT else (k, m)
        br, bc = (k, n) if tb == NT else (n, k)
        A = g.uniform(-1, 1, ar * ac).astype(np.float32)
        B = g.uniform(-1, 1, br * bc).astype(np.float32)
        Cm = g.uniform(-1, 1, m * n).astype(np.float32)
        cases.append(Case("sgemm", [ROW, ta, tb, m, n, k, 1.25, A, ac, B, bc, -0.5, Cm, n], [12], nred=k + 1))
    return cases


@pytest.mark.gpu
def test_tensor_core_group_matches_split_bf16_sgemm(cuda):
    """Calls of at least 128 in m, n and k run in the grouped tensor-core
    product and give exo_sgemm's split-BF16 bits; the others stay on the
    FFMA units; every call within the FP32 bound; with the tensor cores
    switched off no call goes there."""
    import exoblas_gb300 as eb
    from exoblas_gb300 import batch

    torch = cuda
    cases = _tc_cases()
    eligible = [c.args[3] >= 128 and c.args[4] >= 128 and c.args[5] >= 128 for c in cases]
    ops, dev = _to_ops(torch, cases)
    plan = batch.BatchPlan(ops)
    assert plan.tensor_core_calls() == sum(eligible)
    plan.run()
    torch.cuda.synchronize()
    outs = [d[12].cpu().numpy() for d in dev]
    plan.close()
    for c, got, tc in zip(cases, outs, eligible):
        _check(c, got)
        if tc:
            # the same call alone on the split-BF16 path
            a = [torch.from_numpy(v.copy()).cuda() if isinstance(v, np.ndarray) else v for v in c.args]
            eb.set_precision(eb.PRECISION_SPLIT_BF16)
            try:
                eb.exo_sgemm(*a)
            finally:
                eb.set_precision(eb.PRECISION_NATIVE)
            assert a[12].cpu().numpy().tobytes() == got.tobytes(), f"{c.args[3:6]}: group differs from exo_sgemm"
    batch.set_tensor_cores(False)
    try:
        ops2, _ = _to_ops(torch, cases)
        plan2 = batch.BatchPlan(ops2)
        assert plan2.tensor_core_calls() == 0
        plan2.close()
    finally:
        batch.set_tensor_cores(True)


@pytest.mark.gpu
def test_graph_launch_first_on_a_fresh_thread(cuda):
    """A plan whose first use is a graph launch, on a thread that has not
    called the library before (nothing allocated yet in its context): the
    capture must not allocate, and the replay equals a plain run."""
    import threading

    from exoblas_gb300 import batch

    torch = cuda
    cases = _tc_cases(seed=5)[:4]
    ops, dev = _to_ops(torch, cases)
    box = {}

    def body():
        try:
            torch.cuda.set_device(0)
            plan = batch.BatchPlan(ops)
            plan.graph_launch()
            torch.cuda.synchronize()
            box["graph"] = [d[12].clone() for d in dev]
            plan.run()
            torch.cuda.synchronize()
            box["run"] = [d[12].clone() for d in dev]
            plan.close()
        except Exception as e:  # reported on the main thread
            box["error"] = e

    t = threading.Thread(target=body)
    t.start()
    t.join()
    assert "error" not in box, box.get("error")
    for c, g in zip(cases, box["graph"]):
        _check(c, g.cpu().numpy())
