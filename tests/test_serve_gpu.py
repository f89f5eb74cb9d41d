"""Request server with continuous batching: every request of a mixed stream
(gemm / gemv / trsv / syrk, single and double precision, served on several
worker streams at once) must give the same bits as the same request served
alone, and meet the oracle checks (1% rule and componentwise FP bound, trsv
by the residual bound)."""
import numpy as np
import pytest

from common import LO, NT, NU, ROW, TR, UN, UP, Case, assert_rel1pct, check_case, run_oracle, trsv_residual_ok

DT = {"s": np.float32, "d": np.float64}


def _cases(seed=21, count=48, hi=400):
    g = np.random.default_rng(seed)
    out = []
    for i in range(count):
        kind = ("gemm", "gemv", "trsv", "syrk")[i % 4]
        p = "sd"[(i // 4) % 2]
        dt = DT[p]
        m, n, k = (int(v) for v in np.exp(g.uniform(np.log(8), np.log(hi), 3)).astype(int))
        if kind == "gemm":
            ta, tb = (NT, TR)[(i // 8) % 2], (NT, TR)[(i // 16) % 2]
            ar, ac = (m, k) if ta == NT else (k, m)
            br, bc = (k, n) if tb == NT else (n, k)
            A, B = g.uniform(-1, 1, ar * ac).astype(dt), g.uniform(-1, 1, br * bc).astype(dt)
            Cm = g.uniform(-1, 1, m * n).astype(dt)
            out.append(Case(p + "gemm", [ROW, ta, tb, m, n, k, 1.5, A, ac, B, bc, 0.5, Cm, n], [12], nred=k + 1))
        elif kind == "gemv":
            t = (NT, TR)[(i // 8) % 2]
            incx, incy = (1, 2, -1)[i % 3], (1, -2)[(i // 8) % 2]
            xl, yl = (n, m) if t == NT else (m, n)
            A = g.uniform(-1, 1, m * n).astype(dt)
            x = g.uniform(-1, 1, 1 + (xl - 1) * abs(incx)).astype(dt)
            y = g.uniform(-1, 1, 1 + (yl - 1) * abs(incy)).astype(dt)
            out.append(Case(p + "gemv", [ROW, t, m, n, 0.75, A, n, x, incx, 0.5, y, incy], [10], nred=xl + 1))
        elif kind == "trsv":
            u, t, d = (UP, LO)[(i // 8) % 2], (NT, TR)[(i // 16) % 2], (NU, UN)[(i // 32) % 2]
            A = g.uniform(-1, 1, (m, m)) / m
            A[np.arange(m), np.arange(m)] = 1 + g.uniform(0, 1, m)
            x = g.uniform(-1, 1, m)
            out.append(Case(p + "trsv", [ROW, u, t, d, m, A.astype(dt).ravel(), m, x.astype(dt), 1], [7],
                            nred=m + 1))
        else:
            u, t = (UP, LO)[(i // 8) % 2], (NT, TR)[(i // 16) % 2]
            ar, ac = (m, k) if t == NT else (k, m)
            A = g.uniform(-1, 1, ar * ac).astype(dt)
            Cm = g.uniform(-1, 1, m * m).astype(dt)
            out.append(Case(p + "syrk", [ROW, u, t, m, k, 13.0, A, ac, 18.0, Cm, m], [9], nred=k + 1))
    return out


def _requests(torch, cases):
    from exoblas_gb300 import serve as sv

    reqs, dev = [], []
    for c in cases:
        a = [torch.from_numpy(v.copy()).cuda() if isinstance(v, np.ndarray) else v for v in c.args]
        dev.append(a)
        prec = sv.SINGLE if c.op[0] == "s" else sv.DOUBLE
        op = c.op[1:]
        if op == "gemm":
            _, ta, tb, m, n, k, al, A, lda, B, ldb, be, Cm, ldc = a
            reqs.append(sv.request(sv.GEMM, prec, (ta, tb), m, n, k, al, be, A, lda, B, ldb, Cm, ldc))
        elif op == "gemv":
            _, t, m, n, al, A, lda, x, ix, be, y, iy = a
            reqs.append(sv.request(sv.GEMV, prec, (t,), m, n, 0, al, be, A, lda, x, ix, y, iy))
        elif op == "trsv":
            _, u, t, d, n, A, lda, x, ix = a
            reqs.append(sv.request(sv.TRSV, prec, (u, t, d), n, 0, 0, 1.0, 0.0, A, lda, None, 0, x, ix))
        else:
            _, u, t, n, k, al, A, lda, be, Cm, ldc = a
            reqs.append(sv.request(sv.SYRK, prec, (u, t), n, 0, k, al, be, A, lda, None, 0, Cm, ldc))
    torch.cuda.synchronize()
    return reqs, dev


def _outputs(cases, dev):
    return [d[c.outputs[0]].cpu().numpy().copy() for c, d in zip(cases, dev)]


@pytest.mark.gpu
@pytest.mark.parametrize("hi", [400, 1500])
def test_served_results_same_alone_and_in_mix(cuda, hi):
    """hi = 400: nearly every request is small enough for the device
    batches; hi = 1500: the mix straddles the size thresholds, so device
    batches and worker streams run side by side."""
    from exoblas_gb300 import serve as sv

    torch = cuda
    cases = _cases(hi=hi)
    # alone: one request at a time, each drained before the next is submitted
    reqs, dev = _requests(torch, cases)
    s = sv.Server(workers=4)
    for r in reqs:
        s.submit(r)
        s.drain()
    alone = _outputs(cases, dev)
    st = s.stats()
    assert st["completed"] == len(cases) and st["failed"] == 0 and st["rejected"] == 0
    s.close()
    # in the mix: all requests at once on 8 workers (fresh operands)
    reqs, dev = _requests(torch, cases)
    s = sv.Server(workers=8)
    s.replay(reqs, [0.0] * len(reqs))
    s.drain()
    mixed = _outputs(cases, dev)
    st = s.stats()
    assert st["completed"] == len(cases) and st["failed"] == 0
    assert st["p99_s"] >= st["p50_s"] > 0
    bs = s.batch_stats()
    assert bs["batched"] > 0 and bs["batches"] >= 1  # small requests went through device batches
    s.close()
    for i, c in enumerate(cases):
        assert alone[i].tobytes() == mixed[i].tobytes(), f"request {i} ({c}) differs alone vs in the mix"
        got = c.clone_args()
        got[c.outputs[0]] = mixed[i]
        if c.op.endswith("trsv"):
            _, o_a = run_oracle(c)
            assert_rel1pct(mixed[i], o_a[c.outputs[0]], f"served {c}")
            trsv_residual_ok(c, mixed[i])
        else:
            check_case(c, None, got, what="served")


@pytest.mark.gpu
def test_server_admission_and_poisson_replay(cuda):
    """A request whose workspace cannot fit the budget is rejected and
    counted; a Poisson replay of a small mixed stream completes."""
    from exoblas_gb300 import serve as sv
    from exoblas_gb300 import workloads

    torch = cuda
    s = sv.Server(workers=2, hbm_budget=1 << 20)
    A = torch.rand(512 * 512, dtype=torch.float64, device="cuda")
    Cm = torch.zeros(512 * 512, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    s.submit(sv.request(sv.GEMM, sv.DOUBLE, (111, 111), 512, 512, 512, 1.0, 0.0, A, 512, A, 512, Cm, 512))
    s.drain()
    st = s.stats()
    assert st["rejected"] == 1 and st["completed"] == 0
    s.close()

    stream = workloads.serve_stream(200, rate=20000.0, hi=512)
    ops = workloads.ServeOperands(torch, in_elems=(1 << 22, 1 << 21), out_elems=(1 << 22, 1 << 21), hi=512)
    reqs = [ops.request(op, p, m, n, k)[0] for (_, op, p, m, n, k) in stream]
    torch.cuda.synchronize()
    s = sv.Server(workers=4)
    s.replay(reqs, [e[0] for e in stream])
    s.drain()
    st = s.stats()
    assert st["completed"] == 200 and st["failed"] == 0
    assert st["solves_per_s"] > 0
    for t in list(ops.out.values()):
        assert torch.isfinite(t).all()
    s.close()
