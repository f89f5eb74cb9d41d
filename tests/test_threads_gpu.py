"""Concurrent calls from several host threads.  Every thread has its own
stream, scratch and staging buffers (the reference's level-3 procs, with
their static pack buffers, are not re-entrant), and every kernel reduces in
a fixed order, so each thread's results must equal the single-threaded
results bit for bit while the other threads run.  ctypes releases the GIL
for the duration of each call, so the calls really overlap."""
import threading

import numpy as np
import pytest


def _jobs():
    rng = np.random.default_rng(13)
    jobs = []
    for t in range(8):
        m = 96 + 40 * t
        n = 200 + 30 * t
        L = np.tril(rng.uniform(-1, 1, (n, n)) / n)
        L[np.arange(n), np.arange(n)] = 1 + rng.uniform(0, 1, n)
        jobs.append({
            "A": rng.uniform(-1, 1, (m, m)).astype(np.float32),
            "B": rng.uniform(-1, 1, (m, m)).astype(np.float32),
            "x": rng.uniform(-1, 1, 50000 + 1000 * t).astype(np.float32),
            "y": rng.uniform(-1, 1, 50000 + 1000 * t).astype(np.float32),
            "L": L,
            "b": rng.uniform(-1, 1, n),
        })
    return jobs


def _run(eb, j):
    m = j["A"].shape[0]
    C = np.zeros((m, m), np.float32)
    eb.exo_sgemm(101, 111, 111, m, m, m, 1.0, j["A"], m, j["B"], m, 0.0, C, m)
    d = eb.exo_sdot(j["x"].size, j["x"], 1, j["y"], 1)
    v = np.zeros(m, np.float32)
    eb.exo_sgemv(101, 112, m, m, 1.0, j["A"], m, j["B"][0], 1, 0.0, v, 1)
    n = j["b"].size
    s = j["b"].copy()
    eb.exo_dtrsv(101, 122, 111, 131, n, j["L"], n, s, 1)
    return C, np.float32(d), v, s


@pytest.mark.gpu
def test_concurrent_threads_give_single_thread_bits(cuda):
    import exoblas_gb300 as eb

    jobs = _jobs()
    ref = [_run(eb, j) for j in jobs]
    errors = []

    def worker(i):
        try:
            for _ in range(4):
                got = _run(eb, jobs[i])
                for a, b in zip(got, ref[i]):
                    if np.asarray(a).tobytes() != np.asarray(b).tobytes():
                        errors.append(f"thread {i}: result differs")
                        return
                if eb.status() != 0:
                    errors.append(f"thread {i}: status {eb.status()}")
                    return
        except Exception as e:  # surfaced below
            errors.append(f"thread {i}: {e!r}")

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(len(jobs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not any(t.is_alive() for t in threads), "a thread did not finish"
    assert not errors, errors
