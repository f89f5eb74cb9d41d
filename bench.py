#!/usr/bin/env python
"""Benchmark of the ExoBLAS hot path on GB300 through libexoblas_gb300.so.

Workload (one "step"): the level-1/2 bandwidth set, each kernel once over
its own seeded inputs resident in HBM --
  saxpy, sdot, dsdot   n = 2^26 fp32
  daxpy, ddot          n = 2^25 fp64
  sgemv N, sgemv T     M = N = 16384 fp32
  dtrsv                lower / no-trans / non-unit, n = 8192 fp64,
                       off-diagonal uniform[-1,1)/n, diagonal 1 + uniform[0,1)
Every operand is larger than L2 (129 MB) and each kernel has its own buffers,
so no kernel re-reads what another left in L2.

value      aggregate algorithmic GB/s (decimal) of the set, device-resident
           operands, kernels queued through the exo_* C ABI with device
           pointers (non-blocking mode, device-result reductions), timed with
           CUDA events on the library's stream.
e2e        the same set through the same entry points with pageable HOST
           buffers (what a drop-in CBLAS caller passes): the library stages
           every operand host->device and copies outputs back inside the
           timed region (wall clock per step, median step; the mean over the
           run is reported beside it).  The pinned-buffer figure sits beside
           it with this box's pinned copy rates and frac_of_link_bound: the
           time the copies alone (at those rates) plus the device step take,
           over the measured pinned e2e step.
roofline   the kernel with the largest share of the step, against the
           measured HBM copy bandwidth in MEASURED_PEAKS.json.
cpu_baseline  the CPU oracle (C++ restatement of the reference algorithms,
           threaded over ranges/rows) on the full set, all host cores,
           measured by the --impl reference routine in a fresh process.
cpu_openblas  the same set through SciPy's bundled OpenBLAS, the CBLAS the
           reference compares against: one thread and all host threads.
level3     configurations 1 and 3 measured in the same run: sgemm NN 1024^3
           (alpha 1, beta 0.5, seed 0) with the oracle's CPU sgemm beside it,
           and sgemm 8192^3 plain FFMA vs split-BF16 with their errors.

--impl reference times that CPU implementation alone on the host cores:
at least 1 s of warm-up, at least 1 s timed, the median pass.
Multi-GPU: replicas only (one independent replica per rank, no collective).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "gemm TFLOP/s, gemv/trsv HBM GB/s vs roofline; served solves/s, p99 at equal error"
UNIT = "GB/s"
WORKLOAD = "level-1/2 bandwidth set: saxpy/sdot/dsdot n=2^26 f32, daxpy/ddot n=2^25 f64, sgemv N+T 16384^2 f32, dtrsv L/N/NonUnit n=8192 f64"

# algorithmic bytes per call (decimal units in the output)
N1S, N1D, NG, NT = 1 << 26, 1 << 25, 16384, 8192
KERNELS = [
    ("saxpy", 3 * 4 * N1S),
    ("sdot", 2 * 4 * N1S),
    ("dsdot", 2 * 4 * N1S),
    ("daxpy", 3 * 8 * N1D),
    ("ddot", 2 * 8 * N1D),
    ("sgemv_n", (NG * NG + NG + 2 * NG) * 4),
    ("sgemv_t", (NG * NG + NG + 2 * NG) * 4),
    ("dtrsv", (NT * (NT + 1) // 2 + 2 * NT) * 8),
]
BYTES = dict(KERNELS)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-level3", action="store_true", help="skip the level-3 figures of the default line")
    ap.add_argument("--workload", choices=["bandwidth", "precision", "batch", "serve", "routines"],
                    default="bandwidth",
                    help="bandwidth: the level-1/2 set (default); precision: the level-3 precision set; batch: "
                         "4096 mixed instances in one persistent launch; serve: a Poisson request stream; "
                         "routines: every other level-1/2 routine at HBM-sized operands")
    ap.add_argument("--requests", type=int, default=20000, help="serve: requests in the stream")
    ap.add_argument("--rate", type=float, default=20000.0, help="serve: mean arrivals per second")
    ap.add_argument("--workers", type=int, default=8, help="serve: server worker streams")
    ap.add_argument("--per-call-sample", type=int, default=2000, help="serve: requests timed per call")
    ap.add_argument("--size", type=int, default=8192, help="M = N = K of the precision set")
    ap.add_argument("--kernels", default="",
                    help="bandwidth / routines: comma list, a subset of the set (profiling runs)")
    return ap.parse_args()


# ------------------------------------------------------------------ peaks --
def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_table():
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return {}
    return {}


# ----------------------------------------------------------------- clocks --
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = [l.split(",") for l in Path(self.file.name).read_text().splitlines() if l.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- workloads --
def make_inputs(torch, dev, names=None):
    g = torch.Generator(device=dev).manual_seed(0)

    def u(n, dt):
        return (torch.rand(n, generator=g, device=dev, dtype=dt) * 2 - 1)

    f, d = torch.float32, torch.float64
    make = {
        "saxpy": lambda: (u(N1S, f), u(N1S, f)),
        "sdot": lambda: (u(N1S, f), u(N1S, f)),
        "dsdot": lambda: (u(N1S, f), u(N1S, f)),
        "daxpy": lambda: (u(N1D, d), u(N1D, d)),
        "ddot": lambda: (u(N1D, d), u(N1D, d)),
        "sgemv_n": lambda: (u(NG * NG, f), u(NG, f), u(NG, f)),
        "sgemv_t": lambda: (u(NG * NG, f), u(NG, f), u(NG, f)),
    }
    X = {k: make[k]() for k in (names or BYTES) if k in make}
    if "dtrsv" in (names or BYTES):
        A = torch.rand(NT, NT, generator=g, device=dev, dtype=d).mul_(2).sub_(1).div_(NT)
        idx = torch.arange(NT, device=dev)
        A[idx, idx] = 1.0 + torch.rand(NT, generator=g, device=dev, dtype=d)
        X["dtrsv"] = (A.reshape(-1), u(NT, d))
    return X


def launchers(L, X, res):
    """Closures that queue each kernel through the C ABI (device pointers)."""
    p = {k: tuple(t.data_ptr() for t in v) for k, v in X.items()}
    r = res.data_ptr()
    vp = C.c_void_p
    return {
        "saxpy": lambda: L.exo_saxpy(N1S, 0.75, vp(p["saxpy"][0]), 1, vp(p["saxpy"][1]), 1),
        "sdot": lambda: L.exoblas_sdot_device(N1S, vp(p["sdot"][0]), 1, vp(p["sdot"][1]), 1, vp(r)),
        "dsdot": lambda: L.exoblas_dsdot_device(N1S, vp(p["dsdot"][0]), 1, vp(p["dsdot"][1]), 1, vp(r + 8)),
        "daxpy": lambda: L.exo_daxpy(N1D, 0.75, vp(p["daxpy"][0]), 1, vp(p["daxpy"][1]), 1),
        "ddot": lambda: L.exoblas_ddot_device(N1D, vp(p["ddot"][0]), 1, vp(p["ddot"][1]), 1, vp(r + 16)),
        "sgemv_n": lambda: L.exo_sgemv(101, 111, NG, NG, 1.0, vp(p["sgemv_n"][0]), NG, vp(p["sgemv_n"][1]), 1, 0.5,
                                       vp(p["sgemv_n"][2]), 1),
        "sgemv_t": lambda: L.exo_sgemv(101, 112, NG, NG, 1.0, vp(p["sgemv_t"][0]), NG, vp(p["sgemv_t"][1]), 1, 0.5,
                                       vp(p["sgemv_t"][2]), 1),
        "dtrsv": lambda: L.exo_dtrsv(101, 122, 111, 131, NT, vp(p["dtrsv"][0]), NT, vp(p["dtrsv"][1]), 1),
    }


def host_launchers(L, H):
    """Same calls with pinned host buffers (staged by the library)."""
    p = {k: tuple(t.data_ptr() for t in v) for k, v in H.items()}
    vp = C.c_void_p
    return {
        "saxpy": lambda: L.exo_saxpy(N1S, 0.75, vp(p["saxpy"][0]), 1, vp(p["saxpy"][1]), 1),
        "sdot": lambda: L.exo_sdot(N1S, vp(p["sdot"][0]), 1, vp(p["sdot"][1]), 1),
        "dsdot": lambda: L.exo_dsdot(N1S, vp(p["dsdot"][0]), 1, vp(p["dsdot"][1]), 1),
        "daxpy": lambda: L.exo_daxpy(N1D, 0.75, vp(p["daxpy"][0]), 1, vp(p["daxpy"][1]), 1),
        "ddot": lambda: L.exo_ddot(N1D, vp(p["ddot"][0]), 1, vp(p["ddot"][1]), 1),
        "sgemv_n": lambda: L.exo_sgemv(101, 111, NG, NG, 1.0, vp(p["sgemv_n"][0]), NG, vp(p["sgemv_n"][1]), 1, 0.5,
                                       vp(p["sgemv_n"][2]), 1),
        "sgemv_t": lambda: L.exo_sgemv(101, 112, NG, NG, 1.0, vp(p["sgemv_t"][0]), NG, vp(p["sgemv_t"][1]), 1, 0.5,
                                       vp(p["sgemv_t"][2]), 1),
        "dtrsv": lambda: L.exo_dtrsv(101, 122, 111, 131, NT, vp(p["dtrsv"][0]), NT, vp(p["dtrsv"][1]), 1),
    }


# ----------------------------------------------------------- CPU baseline --
# The reference's CPU path on the same workload: the full bandwidth set at the
# sizes above (one pass = every kernel once), seeded uniform[-1, 1) inputs
# generated on the host.  sgemv N and T read one shared matrix (each pass
# streams it twice from DRAM all the same: 1 GiB is far beyond the caches).
CPU_DESC = ("full bandwidth set (saxpy/sdot/dsdot n=2^26, daxpy/ddot n=2^25, sgemv N+T 16384^2, dtrsv n=8192) "
            "through the oracle's threaded drivers (C++ restatement of the reference algorithms, -O3, "
            "std::thread ranges, no pinning)")
CPU_PROTOCOL = ">=1 s warm-up, >=1 s and >=3 passes timed, median pass (test/CMakeLists.txt:49-57)"


def cpu_inputs():
    import numpy as np

    g = np.random.default_rng(0)

    def u(n, dt):
        v = g.random(n, dtype=dt)
        v *= 2
        v -= 1
        return v

    f, d = np.float32, np.float64
    S = {"saxpy": (u(N1S, f), u(N1S, f)), "sdot": (u(N1S, f), u(N1S, f)), "dsdot": (u(N1S, f), u(N1S, f)),
         "daxpy": (u(N1D, d), u(N1D, d)), "ddot": (u(N1D, d), u(N1D, d))}
    Ag = u(NG * NG, f)
    S["sgemv_n"] = (Ag, u(NG, f), u(NG, f))
    S["sgemv_t"] = (Ag, u(NG, f), u(NG, f))
    A = u(NT * NT, d).reshape(NT, NT)
    A /= NT
    A[np.arange(NT), np.arange(NT)] = 1.0 + g.random(NT)
    S["dtrsv"] = (A.ravel(), u(NT, d))
    return S


def cpu_pass(S, threads):
    """One pass of the set through the oracle's threaded drivers (threads > 0)
    or through OpenBLAS (threads = 0, its own thread setting); returns seconds."""
    import oracle

    t0 = time.perf_counter()
    for k, _ in KERNELS:
        a = S[k]
        if threads <= 0:
            from oracle import cblas

            if k in ("saxpy", "daxpy"):
                cblas.call(k, len(a[0]), 0.75, a[0], 1, a[1], 1)
            elif k in ("sdot", "ddot", "dsdot"):
                cblas.call(k, len(a[0]), a[0], 1, a[1], 1)
            elif k in ("sgemv_n", "sgemv_t"):
                cblas.call("sgemv", 101, 111 if k == "sgemv_n" else 112, NG, NG, 1.0, a[0], NG, a[1], 1, 0.5, a[2], 1)
            else:
                x = a[1].copy()
                cblas.call("dtrsv", 101, 122, 111, 131, NT, a[0], NT, x, 1)
            continue
        if k == "saxpy":
            oracle.call("par_saxpy", threads, N1S, 0.75, a[0], a[1])
        elif k == "daxpy":
            oracle.call("par_daxpy", threads, N1D, 0.75, a[0], a[1])
        elif k == "sdot":
            oracle.call("par_sdot", threads, N1S, a[0], a[1])
        elif k == "ddot":
            oracle.call("par_ddot", threads, N1D, a[0], a[1])
        elif k == "dsdot":
            oracle.call("par_dsdot", threads, N1S, a[0], a[1])
        elif k in ("sgemv_n", "sgemv_t"):
            oracle.call("par_sgemv", threads, 111 if k == "sgemv_n" else 112, NG, NG, 1.0, a[0], NG, a[1], 0.5, a[2])
        else:
            x = a[1].copy()
            oracle.call("par_dtrsv_lnn", threads, NT, a[0], NT, x)
    return time.perf_counter() - t0


def cpu_measure(S, threads, warm_passes=0, passes=0, warm_s=1.0, min_s=1.0):
    """The reference's benchmark protocol on the host: warm up for at least
    warm_s (and warm_passes passes), then time passes until at least min_s
    and max(passes, 3) passes have run; GB/s of the median pass."""
    t, w = 0.0, 0
    while t < warm_s or w < warm_passes:
        t += cpu_pass(S, threads)
        w += 1
    times = []
    while sum(times) < min_s or len(times) < max(passes, 3):
        times.append(cpu_pass(S, threads))
    step_bytes = sum(BYTES.values())
    med = statistics.median(times)
    return {"value": round(step_bytes / med / 1e9, 3), "ms_per_pass": round(med * 1e3, 3), "passes": len(times),
            "warmup_passes": w, "seconds": round(sum(times), 2),
            "spread": [round(step_bytes / max(times) / 1e9, 3), round(step_bytes / min(times) / 1e9, 3)]}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline():
    """The reference arm's own measurement (same routine, same sizes), run in
    a fresh process so that it sees the host exactly as `--impl reference`
    does (no CUDA context, no pinned buffers of this process)."""
    r = subprocess.run([sys.executable, str(Path(__file__).resolve()), "--impl", "reference", "--steps", "3",
                        "--warmup", "1"], capture_output=True, text=True)
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    if r.returncode != 0 or not lines:
        return {"unavailable": f"reference arm exited {r.returncode}: {r.stderr.strip()[-300:]}"}
    ref = json.loads(lines[-1])
    return dict(ref["cpu_baseline"], ms_per_pass=ref["ms_per_step"], same_config=True)


def host_link_rates(local, nbytes=1 << 30):
    """Pinned host <-> device copy rates (GB/s) of this box, 1 GiB each way."""
    import torch

    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device=f"cuda:{local}")
    out = []
    for src, dst in ((h, d), (d, h)):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        out.append(3 * nbytes / (time.perf_counter() - t0) / 1e9)
    del h, d
    return out[0], out[1]


def openblas_baseline(S=None):
    """The same full set through SciPy's bundled OpenBLAS (the CBLAS the
    reference compares against), one thread and all host threads, with the
    same protocol as cpu_measure."""
    try:
        from oracle import cblas

        if not cblas.available():
            return {"unavailable": "SciPy's bundled OpenBLAS not found"}
    except ImportError as e:
        return {"unavailable": f"oracle.cblas: {e}"}
    S = S or cpu_inputs()
    cores = cpu_threads()
    out = {"unit": UNIT, "kind": "OpenBLAS bundled with SciPy (scipy_cblas_*)", "sample": "full bandwidth set",
           "protocol": CPU_PROTOCOL, "cores": cores}
    for label, threads in (("one_thread", 1), ("all_threads", cores)):
        cblas.set_threads(threads)
        out[label] = cpu_measure(S, 0)["value"]
    cblas.set_threads(1)
    return out


# --------------------------------------------------------------- replicas --
def max_over_ranks(dist, value, device):
    """The largest `value` over all ranks (the replicas' slowest time).  The
    bench's GPU ranks pass a CUDA device (NCCL); the same host logic runs
    over gloo with device "cpu" in the multi-process CPU tests."""
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------- level-3 figures --
def level3_figures(L, eb, torch, stream, cpu=True):
    """Level-3 configurations measured beside the bandwidth set.

    sgemm_1024: sgemm NN 1024^3, lda = ldb = ldc = 1024, alpha 1, beta 0.5, A,
    B, C uniform[-1, 1) from seed 0 (NumPy PCG64, float64 cast to float32):
    device TFLOP/s over 2MNK + 3MN flops (CUDA events, mean of 50 calls after
    5), the max / median componentwise relative error of one call against
    FP64, and the oracle's sgemm (the reference algorithm, one thread and all
    host threads) on the same inputs.
    sgemm_8192: sgemm NN 8192^3 uniform[-1, 1), plain FP32 FFMA and
    split-BF16 on tcgen05, TFLOP/s and error on 128 sampled rows against an
    FP64 product on the device."""
    import numpy as np

    vp = C.c_void_p

    def timed(fn, warm, reps):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        if L.exoblas_synchronize() != 0:
            raise RuntimeError("library failure in the level-3 figures")
        return e0.elapsed_time(e1) / reps

    def errs(got, ref, mag):
        rel = ((got - ref).abs() / mag.clamp_min(1e-300)).flatten()
        return {"max_rel_err": float(rel.max()), "median_rel_err": float(rel.median())}

    out = {}
    n = 1024
    g = np.random.default_rng(0)
    A = g.uniform(-1, 1, (n, n)).astype(np.float32)
    B = g.uniform(-1, 1, (n, n)).astype(np.float32)
    C0 = g.uniform(-1, 1, (n, n)).astype(np.float32)
    dA, dB, dC0 = (torch.from_numpy(v).cuda() for v in (A, B, C0))
    dC = dC0.clone()
    torch.cuda.synchronize()
    f = lambda: L.exo_sgemm(101, 111, 111, n, n, n, 1.0, vp(dA.data_ptr()), n, vp(dB.data_ptr()), n, 0.5,
                            vp(dC.data_ptr()), n)
    ms = timed(f, 5, 50)
    dC.copy_(dC0)
    torch.cuda.synchronize()
    timed(f, 0, 1)
    A64, B64, C64 = dA.double(), dB.double(), dC0.double()
    flops1 = 2.0 * n ** 3 + 3.0 * n * n
    out["sgemm_1024"] = {"config": "sgemm NN 1024^3 alpha 1 beta 0.5 seed 0", "ms": round(ms, 4),
                         "tflops": round(flops1 / ms / 1e9, 2),
                         **errs(dC.double(), A64 @ B64 + 0.5 * C64, A64.abs() @ B64.abs() + 0.5 * C64.abs())}
    if cpu:
        import oracle

        threads = cpu_threads()
        for label, th in (("cpu_port_one_thread", 1), ("cpu_port_all_threads", threads)):
            Cc = C0.copy()
            oracle.call("par_sgemm", th, 111, 111, n, n, n, 1.0, A, n, B, n, 0.5, Cc, n)  # warm-up
            ts = []
            while sum(ts) < 1.0 or len(ts) < 3:
                Cc = C0.copy()
                t0 = time.perf_counter()
                oracle.call("par_sgemm", th, 111, 111, n, n, n, 1.0, A, n, B, n, 0.5, Cc, n)
                ts.append(time.perf_counter() - t0)
            med = statistics.median(ts)
            out["sgemm_1024"][label] = {"ms": round(med * 1e3, 2), "tflops": round(flops1 / med / 1e12, 4),
                                        "threads": th}
    del dA, dB, dC, dC0, A64, B64, C64

    n = 8192
    gen = torch.Generator(device="cuda").manual_seed(0)
    A = (torch.rand(n, n, device="cuda", generator=gen, dtype=torch.float64) * 2 - 1).float()
    B = (torch.rand(n, n, device="cuda", generator=gen, dtype=torch.float64) * 2 - 1).float()
    rows = torch.arange(0, n, n // 128, device="cuda")
    Ar, B64 = A[rows].double(), B.double()
    ref, mag = Ar @ B64, Ar.abs() @ B64.abs()
    del B64
    res = {}
    for mode, name in ((eb.PRECISION_NATIVE, "ffma"), (eb.PRECISION_SPLIT_BF16, "split_bf16")):
        eb.set_precision(mode)
        try:
            Cg = torch.zeros(n, n, device="cuda")
            f = lambda: L.exo_sgemm(101, 111, 111, n, n, n, 1.0, vp(A.data_ptr()), n, vp(B.data_ptr()), n, 0.0,
                                    vp(Cg.data_ptr()), n)
            ms = timed(f, 1, 3 if mode == eb.PRECISION_NATIVE else 6)
        finally:
            eb.set_precision(eb.PRECISION_NATIVE)
        res[name] = {"ms": round(ms, 3), "tflops": round(2.0 * n ** 3 / ms / 1e9, 1),
                     **errs(Cg[rows].double(), ref, mag)}
        del Cg
    res["speedup_split_over_ffma"] = round(res["split_bf16"]["tflops"] / res["ffma"]["tflops"], 2)
    res["config"] = "sgemm NN 8192^3 uniform[-1,1), alpha 1 beta 0; error on 128 rows against FP64"
    out["sgemm_8192"] = res
    return out


# ------------------------------------------------------------------- main --
def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        return run_reference(args)
    if args.workload == "precision":
        return run_precision(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "routines":
        return run_routines(args)
    if args.workload == "batch":
        return run_batch(args)

    import torch

    import exoblas_gb300 as eb
    from exoblas_gb300 import _native

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    L = _native.lib()
    stream = torch.cuda.Stream()
    eb.set_stream(stream)
    eb.set_blocking(False)

    names = [k for k, _ in KERNELS]
    if args.kernels:
        names = [k for k in names if k in args.kernels.split(",")]
        if not names:
            raise SystemExit(f"--kernels: none of {args.kernels!r} in {[k for k, _ in KERNELS]}")
    X = make_inputs(torch, f"cuda:{local}", names)
    res = torch.zeros(8, dtype=torch.float64, device=f"cuda:{local}")
    torch.cuda.synchronize()  # inputs were generated on the default stream
    run = launchers(L, X, res)

    def step(evs=None):
        for i, k in enumerate(names):
            if evs is not None:
                evs[i][0].record(stream)
            run[k]()
            if evs is not None:
                evs[i][1].record(stream)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    L.exoblas_synchronize()
    if L.exoblas_get_status() != 0:
        raise RuntimeError(f"library status {L.exoblas_get_status()} during warm-up")
    torch.cuda.synchronize()

    K = args.steps
    evs = [[[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)] for _ in names]
           for _ in range(K)]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.25)
    launches0 = eb.kernel_launches()
    t_start.record(stream)
    for s in range(K):
        step(evs[s])
    t_end.record(stream)
    torch.cuda.synchronize()
    launches = eb.kernel_launches() - launches0
    clk = clocks.stop()
    if L.exoblas_synchronize() != 0:
        raise RuntimeError("library reported a failure in the timed region")
    total_ms = t_start.elapsed_time(t_end)
    if dist:
        total_ms = max_over_ranks(dist, total_ms, f"cuda:{local}")
        dist.barrier()

    per = {k: statistics.mean(evs[s][i][0].elapsed_time(evs[s][i][1]) for s in range(K)) for i, k in enumerate(names)}
    step_bytes = sum(BYTES[k] for k in names)
    ms_per_step = total_ms / K
    value = world * step_bytes / (ms_per_step * 1e-3) / 1e9

    hbm, peak_kind = peaks()
    traffic = traffic_table()
    dom = max(per, key=per.get)
    achieved = BYTES[dom] / (per[dom] * 1e-3) / 1e9
    kern = {k: {"ms": round(per[k], 4), "GB/s": round(BYTES[k] / (per[k] * 1e-3) / 1e9, 1),
                "frac_of_measured_hbm": round(BYTES[k] / (per[k] * 1e-3) / 1e9 / hbm, 3),
                "share": round(per[k] / sum(per.values()), 3)} for k in names}

    # ---- end to end through the C ABI with host buffers: pageable memory
    # (what a drop-in CBLAS caller hands over, the headline) and pinned
    # memory (reported beside it)
    e2e = None
    if not args.no_e2e:
        eb.set_blocking(True)

        def e2e_run(H):
            hrun = host_launchers(L, H)
            for k in names:
                hrun[k]()
            h0, d0 = C.c_ulonglong(), C.c_ulonglong()
            h1, d1 = C.c_ulonglong(), C.c_ulonglong()
            KE = max(3, min(K, 20))
            if dist:
                dist.barrier()
            torch.cuda.synchronize()
            L.exoblas_staged_bytes(C.byref(h0), C.byref(d0))
            bad = 0
            steps = []
            t0 = time.perf_counter()
            for _ in range(KE):
                ts = time.perf_counter()
                for k in names:
                    hrun[k]()
                    bad |= L.exoblas_get_status()  # each blocking call reports its own status
                torch.cuda.synchronize()
                steps.append(time.perf_counter() - ts)
            t1 = time.perf_counter()
            L.exoblas_staged_bytes(C.byref(h1), C.byref(d1))
            if bad != 0:
                raise RuntimeError("library reported a failure in the e2e region")
            # the median step: the host link is shared with other tenants of
            # the machine, so a mean over the run can carry their bursts
            med = statistics.median(steps)
            mean = (t1 - t0) / KE
            if dist:
                med = max_over_ranks(dist, med, f"cuda:{local}")
                mean = max_over_ranks(dist, mean, f"cuda:{local}")
            return med, mean, KE, (h1.value - h0.value) // KE, (d1.value - d0.value) // KE

        Hpage = {k: tuple(t.cpu() for t in v) for k, v in X.items()}
        e2e_med, e2e_mean, KE, h2d_step, d2h_step = e2e_run(Hpage)
        del Hpage
        Hpin = {k: tuple(t.cpu().pin_memory() for t in v) for k, v in X.items()}
        pin_med, pin_mean, KP, _, _ = e2e_run(Hpin)
        del Hpin
        link_h, link_d = host_link_rates(local)
        # time the pinned host link alone would need per step (copies in,
        # device work, copies out, one after another) over the measured step
        ideal = h2d_step / (link_h * 1e9) + d2h_step / (link_d * 1e9) + ms_per_step * 1e-3
        gbs = lambda t: round(world * step_bytes / t / 1e9, 2)
        e2e = {"value": gbs(e2e_med), "unit": UNIT, "statistic": "median step", "mean_over_run": gbs(e2e_mean),
               "h2d_bytes_per_step": h2d_step, "d2h_bytes_per_step": d2h_step, "steps": KE,
               "host_memory": "pageable (torch CPU tensors, malloc-backed)",
               "pinned": {"value": gbs(pin_med), "mean_over_run": gbs(pin_mean), "steps": KP,
                          "frac_of_link_bound": round(ideal / pin_med, 3)},
               "link_h2d_gbs": round(link_h, 1), "link_d2h_gbs": round(link_d, 1)}

    level3 = None
    if rank == 0 and not args.no_level3:
        with torch.cuda.stream(stream):
            level3 = level3_figures(L, eb, torch, stream, cpu=not args.no_cpu_baseline)

    cpu = openblas = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline()
        openblas = openblas_baseline()

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": round(value, 2),
            "unit": UNIT,
            "n_gpus": world,
            "steps": K,
            "warmup": args.warmup,
            "ms_per_step": round(ms_per_step, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32+f64",
            "data": "synthetic (seeded uniform[-1,1); dtrsv off-diagonal uniform/n, diagonal 1+uniform[0,1))",
            "config": {"workload": WORKLOAD, "bytes_per_step": step_bytes,
                       "l2": "inputs larger than L2, distinct buffers per kernel (4.6 GB touched per step)",
                       "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": hbm,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / hbm, 3),
                         "traffic": traffic.get(dom)},
            "cpu_baseline": cpu,
            "cpu_openblas": openblas,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk,
            "kernels": kern,
            "level3": level3,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


# ------------------------------------------------------ precision workload --
def run_precision(args):
    """Level-3 precision set (sgemm NN / ssymm Left-Upper / ssyrk Lower-NoTrans
    at size^3 fp32, split-BF16 on tcgen05 vs plain FP32 FFMA; dgemm NN fp64
    native), uniform[-1,1) and the stress set (sign * U[1,2) * 2^e, e in
    [-16, 16]).  Reports TFLOP/s (device time, CUDA events) and the max and
    median componentwise relative error against an FP64 product computed on
    the GPU (torch float64 matmul)."""
    import torch

    import exoblas_gb300 as eb
    from exoblas_gb300 import _native

    L = _native.lib()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    eb.set_stream(stream)
    eb.set_blocking(False)
    n = args.size
    vp = C.c_void_p
    out = {}

    def draw(seed, stress, dtype=torch.float32):
        g = torch.Generator(device="cuda").manual_seed(seed)
        if not stress:
            return (torch.rand(n, n, device="cuda", generator=g, dtype=torch.float64) * 2 - 1).to(dtype)
        sign = torch.where(torch.rand(n, n, device="cuda", generator=g) < 0.5, -1.0, 1.0).double()
        mant = 1 + torch.rand(n, n, device="cuda", generator=g, dtype=torch.float64)
        e = torch.randint(-16, 17, (n, n), device="cuda", generator=g).double()
        return (sign * mant * torch.exp2(e)).to(dtype)

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        if L.exoblas_synchronize() != 0:
            raise RuntimeError("library failure in the precision workload")
        return e0.elapsed_time(e1) / reps

    def errs(Cg, ref, mag):
        rel = ((Cg.double() - ref).abs() / mag.clamp_min(1e-300)).flatten()
        return {"max": float(rel.max()), "median": float(rel.median())}

    flops = {"sgemm": 2.0 * n ** 3, "ssymm": 2.0 * n ** 3, "ssyrk": float(n) * (n + 1) * n, "dgemm": 2.0 * n ** 3}
    for stress in (False, True):
        tag = "stress" if stress else "uniform"
        A, B = draw(1 if stress else 0, stress), draw(11 if stress else 10, stress)
        A64, B64 = A.double(), B.double()
        ref_gemm = A64 @ B64
        mag_gemm = A64.abs() @ B64.abs()
        for mode, mname in ((eb.PRECISION_NATIVE, "ffma"), (eb.PRECISION_SPLIT_BF16, "split_bf16")):
            eb.set_precision(mode)
            Cg = torch.zeros(n, n, device="cuda")
            f = lambda: L.exo_sgemm(101, 111, 111, n, n, n, 1.0, vp(A.data_ptr()), n, vp(B.data_ptr()), n, 0.0,
                                    vp(Cg.data_ptr()), n)
            ms = timed(f, 3 if mode == eb.PRECISION_NATIVE else 5)
            out[f"sgemm_{mname}_{tag}"] = {"ms": round(ms, 3), "tflops": round(flops["sgemm"] / ms / 1e9, 1),
                                          **errs(Cg, ref_gemm, mag_gemm)}
            if not stress:
                # ssymm Left Upper (sym(A) from A's upper triangle) and ssyrk Lower NoTrans
                As = torch.triu(A64) + torch.triu(A64, 1).t()
                Cs = torch.zeros(n, n, device="cuda")
                fs = lambda: L.exo_ssymm(101, 141, 121, n, n, 1.0, vp(A.data_ptr()), n, vp(B.data_ptr()), n, 0.0,
                                         vp(Cs.data_ptr()), n)
                ms = timed(fs, 3 if mode == eb.PRECISION_NATIVE else 5)
                out[f"ssymm_{mname}"] = {"ms": round(ms, 3), "tflops": round(flops["ssymm"] / ms / 1e9, 1),
                                         **errs(Cs, As @ B64, As.abs() @ B64.abs())}
                Ck = torch.zeros(n, n, device="cuda")
                fk = lambda: L.exo_ssyrk(101, 122, 111, n, n, 1.0, vp(A.data_ptr()), n, 0.0, vp(Ck.data_ptr()), n)
                ms = timed(fk, 3 if mode == eb.PRECISION_NATIVE else 5)
                lo = torch.tril(torch.ones(n, n, device="cuda", dtype=torch.bool))
                rk, mk = A64 @ A64.t(), A64.abs() @ A64.abs().t()
                # the diagonal sums a_ik^2 (all terms of one sign, no
                # cancellation) reported apart from the rest of the triangle
                dg = torch.eye(n, device="cuda", dtype=torch.bool)
                off = lo & ~dg
                out[f"ssyrk_{mname}"] = {"ms": round(ms, 3), "tflops": round(flops["ssyrk"] / ms / 1e9, 1),
                                         **errs(Ck[lo], rk[lo], mk[lo]),
                                         "diagonal": errs(Ck[dg], rk[dg], mk[dg]),
                                         "off_diagonal": errs(Ck[off], rk[off], mk[off])}
        eb.set_precision(eb.PRECISION_NATIVE)
        del ref_gemm, mag_gemm
    # dgemm: native FP64 DFMA vs Ozaki slice emulation; error on 256 sampled
    # entries against the double-double oracle (CPU)
    import numpy as np

    import oracle

    for stress in (False, True):
        tag = "stress" if stress else "uniform"
        Ad, Bd = draw(20 if not stress else 22, stress, torch.float64), draw(21 if not stress else 23, stress,
                                                                             torch.float64)
        Ah, Bh = Ad.cpu().numpy(), Bd.cpu().numpy()
        g = np.random.default_rng(9)
        rows = g.integers(0, n, 256).astype(np.int64)
        cols = g.integers(0, n, 256).astype(np.int64)
        ref = np.zeros(256)
        oracle.call("dd_gemm_entries", 0, 0, n, 1.0, Ah, n, Bh, n, 0.0, None, n, rows, cols, 256, ref)
        mag = np.einsum("ik,ki->i", np.abs(Ah[rows]), np.abs(Bh[:, cols]))
        for mode, mname in ((eb.PRECISION_NATIVE, "native"), (eb.PRECISION_OZAKI, "ozaki")):
            if mode == eb.PRECISION_NATIVE and stress:
                continue
            eb.set_precision(mode)
            Cd = torch.zeros(n, n, device="cuda", dtype=torch.float64)
            fd = lambda: L.exo_dgemm(101, 111, 111, n, n, n, 1.0, vp(Ad.data_ptr()), n, vp(Bd.data_ptr()), n, 0.0,
                                     vp(Cd.data_ptr()), n)
            ms = timed(fd, 1 if mode == eb.PRECISION_NATIVE else 3)
            got = Cd.cpu().numpy()[rows, cols]
            rel = np.abs(got - ref) / mag
            out[f"dgemm_{mname}_{tag}"] = {"ms": round(ms, 3), "tflops": round(flops["dgemm"] / ms / 1e9, 2),
                                           "max": float(rel.max()), "median": float(np.median(rel))}
        eb.set_precision(eb.PRECISION_NATIVE)
    line = {
        "metric": METRIC, "unit": "TFLOP/s", "workload": f"level-3 precision set {n}^3",
        "value": out.get("sgemm_split_bf16_uniform", {}).get("tflops"),
        "speedup_split_over_ffma": round(out["sgemm_split_bf16_uniform"]["tflops"] / out["sgemm_ffma_uniform"]["tflops"], 2),
        "speedup_ozaki_over_dfma": round(out["dgemm_ozaki_uniform"]["tflops"] / out["dgemm_native_uniform"]["tflops"], 2),
        "results": out,
    }
    print(json.dumps(line))
    return 0


# ------------------------------------------------------- routines workload --
def run_routines(args):
    """Every level-1 / level-2 routine outside the bandwidth set, each on its
    own device-resident operands larger than L2, timed alone with CUDA events
    on the library's stream (mean over args.steps calls after args.warmup):
    algorithmic bytes (each operand element read or written once) per call
    over the call's time, against the measured HBM copy bandwidth.  Level 1
    at n = 2^26 (f32) / 2^25 (f64); dense level 2 at 16384^2 (f32) /
    11585^2 (f64, same bytes); banded level 2 at 2^21 rows, 32 off-diagonals
    on each side (gbmv) or one side (sbmv, tbmv)."""
    import torch

    import exoblas_gb300 as eb
    from exoblas_gb300 import _native

    L = _native.lib()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    eb.set_stream(stream)
    eb.set_blocking(False)
    g = torch.Generator(device="cuda").manual_seed(3)
    vp = C.c_void_p

    def u(nel, dt):
        return torch.rand(int(nel), generator=g, device="cuda", dtype=dt).mul_(2).sub_(1)

    res = torch.zeros(8, dtype=torch.float64, device="cuda")
    r = vp(res.data_ptr())
    f32, f64 = torch.float32, torch.float64
    items = []  # (name, bytes, closure)

    def level1(p, dt, n, es):
        x, y = u(n, dt), u(n, dt)
        P = torch.tensor([-1.0, 0.9, 0.1, -0.1, 0.9], dtype=dt, device="cuda")
        X, Y, PP = vp(x.data_ptr()), vp(y.data_ptr()), vp(P.data_ptr())
        items.extend([
            (f"{p}asum", es * n, lambda: getattr(L, f"exoblas_{p}asum_device")(n, X, 1, r)),
            (f"{p}copy", 2 * es * n, lambda: getattr(L, f"exo_{p}copy")(n, X, 1, Y, 1)),
            (f"{p}swap", 4 * es * n, lambda: getattr(L, f"exo_{p}swap")(n, X, 1, Y, 1)),
            (f"{p}scal", 2 * es * n, lambda: getattr(L, f"exo_{p}scal")(n, 0.5, X, 1)),
            (f"{p}rot", 4 * es * n, lambda: getattr(L, f"exo_{p}rot")(n, X, 1, Y, 1, 0.8, 0.6)),
            (f"{p}rotm", 4 * es * n, lambda: getattr(L, f"exo_{p}rotm")(n, X, 1, Y, 1, PP)),
        ])
        return x, y, P

    def level2(p, dt, n, es):
        A = u(n * n, dt)
        x, y = u(n, dt), u(n, dt)
        a, X, Y = vp(A.data_ptr()), vp(x.data_ptr()), vp(y.data_ptr())
        tri = n * (n + 1) // 2
        items.extend([
            (f"{p}ger", es * (2 * n * n + 2 * n), lambda: getattr(L, f"exo_{p}ger")(101, n, n, 1e-3, X, 1, Y, 1, a, n)),
            (f"{p}symv", es * (tri + 3 * n),
             lambda: getattr(L, f"exo_{p}symv")(101, 121, n, 1.0, a, n, X, 1, 0.5, Y, 1)),
            (f"{p}syr", es * (2 * tri + n), lambda: getattr(L, f"exo_{p}syr")(101, 122, n, 1e-3, X, 1, a, n)),
            (f"{p}syr2", es * (2 * tri + 2 * n),
             lambda: getattr(L, f"exo_{p}syr2")(101, 121, n, 1e-3, X, 1, Y, 1, a, n)),
            (f"{p}trmv", es * (tri + 2 * n), lambda: getattr(L, f"exo_{p}trmv")(101, 121, 111, 131, n, a, n, X, 1)),
        ])
        return A, x, y

    def banded(p, dt, n, k, es):
        G = u(n * (2 * k + 1), dt)
        B = u(n * (k + 1), dt)
        x, y = u(n, dt), u(n, dt)
        gp, bp, X, Y = vp(G.data_ptr()), vp(B.data_ptr()), vp(x.data_ptr()), vp(y.data_ptr())
        items.extend([
            (f"{p}gbmv", es * (n * (2 * k + 1) + 3 * n),
             lambda: getattr(L, f"exo_{p}gbmv")(n, n, k, k, 1.0, gp, 2 * k + 1, X, 1, 0.5, Y, 1)),
            (f"{p}sbmv", es * (n * (k + 1) + 3 * n),
             lambda: getattr(L, f"exo_{p}sbmv")(101, 121, n, k, 1.0, bp, k + 1, X, 1, 0.5, Y, 1)),
            (f"{p}tbmv", es * (n * (k + 1) + 2 * n),
             lambda: getattr(L, f"exo_{p}tbmv")(101, 121, 111, 131, n, k, bp, k + 1, X, 1)),
        ])
        return G, B, x, y

    want = set(args.kernels.split(",")) if args.kernels else None

    def wanted(*names):
        return want is None or any(nm in want for nm in names)

    keep = []
    for p, dt, es in (("s", f32, 4), ("d", f64, 8)):
        if wanted(*(p + r for r in ("asum", "copy", "swap", "scal", "rot", "rotm"))):
            keep.append(level1(p, dt, (1 << 26) if p == "s" else (1 << 25), es))
        if wanted(*(p + r for r in ("ger", "symv", "syr", "syr2", "trmv"))):
            keep.append(level2(p, dt, 16384 if p == "s" else 11585, es))
        if wanted(*(p + r for r in ("gbmv", "sbmv", "tbmv"))):
            keep.append(banded(p, dt, 1 << 21, 32, es))
    if wanted("snrm2", "isamax", "dnrm2", "idamax"):
        nrm = u(1 << 26, f32), u(1 << 25, f64)
        keep.append(nrm)
        items.append(("snrm2", 4 * (1 << 26), lambda: L.exoblas_snrm2_device(1 << 26, vp(nrm[0].data_ptr()), 1, r)))
        items.append(("isamax", 4 * (1 << 26), lambda: L.exoblas_isamax_device(1 << 26, vp(nrm[0].data_ptr()), 1, r)))
        items.append(("dnrm2", 8 * (1 << 25), lambda: L.exoblas_dnrm2_device(1 << 25, vp(nrm[1].data_ptr()), 1, r)))
        items.append(("idamax", 8 * (1 << 25), lambda: L.exoblas_idamax_device(1 << 25, vp(nrm[1].data_ptr()), 1, r)))
    if want is not None:
        items[:] = [it for it in items if it[0] in want]
    torch.cuda.synchronize()
    hbm, peak_kind = peaks()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    K = max(3, min(args.steps, 50))
    clocks = Clocks(0)
    clocks.start()
    time.sleep(0.25)
    for name, nbytes, fn in items:
        for _ in range(max(args.warmup, 3)):
            fn()
        L.exoblas_synchronize()
        e0.record(stream)
        for _ in range(K):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        if L.exoblas_get_status() != 0:
            raise RuntimeError(f"library status {L.exoblas_get_status()} in {name}")
        ms = e0.elapsed_time(e1) / K
        gbs = nbytes / (ms * 1e-3) / 1e9
        out[name] = {"ms": round(ms, 4), "GB/s": round(gbs, 1), "frac_of_measured_hbm": round(gbs / hbm, 3)}
    clk = clocks.stop()
    tot_b = sum(b for _, b, _ in items)
    tot_ms = sum(v["ms"] for v in out.values())
    line = {
        "metric": METRIC, "unit": UNIT, "value": round(tot_b / (tot_ms * 1e-3) / 1e9, 1), "n_gpus": 1,
        "higher_is_better": True, "dtype": "f32+f64", "data": "synthetic (seeded uniform[-1,1))",
        "config": {"workload": "routines: level-1 (2^26 f32 / 2^25 f64), dense level-2 (16384^2 f32 / 11585^2 f64), "
                               "banded level-2 (2^21 rows, 32 off-diagonals), each call alone", "steps": K},
        "peak": hbm, "peak_kind": peak_kind, "kernels": out, "clocks": clk,
        "note": "reductions write device results (exoblas_*_device), no host synchronisation per call",
    }
    print(json.dumps(line))
    del keep
    return 0


# ---------------------------------------------------------- batch workload --
def run_batch(args):
    """4096 independent sgemm / dgemv / strsv instances (op uniform per
    instance, m, n, k log-uniform in [16, 2048], seed 7) in one persistent
    launch replayed from a CUDA graph, against the same calls issued one at a
    time through the exo_* C ABI (device pointers, non-blocking)."""
    import tempfile as tf

    import torch

    import exoblas_gb300 as eb
    from exoblas_gb300 import _native, batch, workloads

    L = _native.lib()
    torch.cuda.set_device(0)
    os.environ.setdefault("EXOBLAS_TUNE_CACHE", os.path.join(tf.gettempdir(), "exoblas_tune.json"))
    t0 = time.perf_counter()
    batch.tune()
    tune_s = time.perf_counter() - t0
    ops, shapes, arena, views = workloads.batch_config(torch, "cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    eb.set_stream(stream)
    eb.set_blocking(False)
    plan = batch.BatchPlan(ops)
    info = plan.info()
    for _ in range(args.warmup):
        plan.graph_launch()
    torch.cuda.synchronize()
    K = max(3, min(args.steps, 20))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(0)
    clocks.start()
    time.sleep(0.25)
    e0.record(stream)
    for _ in range(K):
        plan.graph_launch()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    batch_ms = e0.elapsed_time(e1) / K
    # the same calls one by one through the C ABI
    vp = C.c_void_p
    calls = []
    for (op, dims, t), o in zip(views, ops):
        if op == "sgemm":
            m, n, k = dims
            calls.append(lambda o=o, m=m, n=n, k=k: L.exo_sgemm(101, 111, 111, m, n, k, 1.0, vp(o.A), k, vp(o.B), n,
                                                                0.5, vp(o.C), n))
        elif op == "dgemv":
            m, n = dims
            calls.append(lambda o=o, m=m, n=n: L.exo_dgemv(101, 111, m, n, 1.0, vp(o.A), n, vp(o.B), 1, 0.5, vp(o.C), 1))
        else:
            (n,) = dims
            calls.append(lambda o=o, n=n: L.exo_strsv(101, 122, 111, 131, n, vp(o.A), n, vp(o.C), 1))
    for f in calls:
        f()
    torch.cuda.synchronize()
    e0.record(stream)
    w0 = time.perf_counter()
    for f in calls:
        f()
    e1.record(stream)
    torch.cuda.synchronize()
    percall_wall_ms = (time.perf_counter() - w0) * 1e3
    percall_ms = e0.elapsed_time(e1)
    plan.close()
    n = len(ops)
    counts = {k: sum(1 for s in shapes if s[0] == k) for k in workloads.OPS}
    line = {
        "metric": METRIC, "workload": "batch: 4096 mixed sgemm/dgemv/strsv, m,n,k log-uniform [16,2048], seed 7",
        "unit": "solves/s", "value": round(n / (batch_ms * 1e-3), 1), "ms_per_batch": round(batch_ms, 3),
        "units": info["units"], "counts": counts,
        "sgemm_gflop": round(info["flops"] / 1e9, 1), "gemv_trsv_gb": round(info["bytes"] / 1e9, 2),
        "effective_tflops": round(info["flops"] / (batch_ms * 1e-3) / 1e12, 2),
        "per_call": {"device_ms": round(percall_ms, 3), "wall_ms": round(percall_wall_ms, 3),
                     "solves_per_s_wall": round(n / (max(percall_ms, percall_wall_ms) * 1e-3), 1)},
        "speedup_vs_per_call": round(max(percall_ms, percall_wall_ms) / batch_ms, 2),
        "autotune_s": round(tune_s, 2), "graph": True, "clocks": clk,
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------- serve workload --
def run_serve(args):
    """A Poisson request stream (mean args.rate req/s, seed 11) of gemm 60% /
    gemv 25% / trsv 10% / syrk 5%, every dimension log-uniform in [32, 8192],
    70% FP32 and 30% FP64 (seed 12), operands resident in HBM, replayed into
    the request server (split-BF16 for FP32 gemm/syrk, Ozaki for FP64
    gemm/syrk, admission by free memory).  Baselines on the first
    args.per_call_sample requests of the same stream, one call after another
    on one stream (blocking calls, as a CPU BLAS user makes them): plain
    per-call launches with the native FFMA / DFMA kernels, and per-call with
    the same precision paths as the server.  The speedups compare those with
    the server replaying the same sample (same requests, same offsets)."""
    import torch

    import exoblas_gb300 as eb
    from exoblas_gb300 import _native, serve, workloads

    L = _native.lib()
    torch.cuda.set_device(0)
    stream = workloads.serve_stream(args.requests, rate=args.rate)
    ops = workloads.ServeOperands(torch, "cuda")
    built = [ops.request(op, p, m, n, k) for (_, op, p, m, n, k) in stream]
    reqs = [b[0] for b in built]
    offsets = [e[0] for e in stream]
    torch.cuda.synchronize()
    work = [workloads.request_work(op, m, n, k, p) for (_, op, p, m, n, k) in stream]
    reserve = int(2.75 * (1 << 30))  # Ozaki workspace of an 8192^3 dgemm, with the arena's growth margin
    W = args.workers
    srv = serve.Server(workers=W, hbm_budget=W * reserve, scratch_reserve=reserve)
    # warm-up: a short stream of small requests through every path
    warm = workloads.serve_stream(400, rate=args.rate, seed_arrivals=3, seed_ops=4, hi=1024)
    wreq = [ops.request(op, p, m, n, k)[0] for (_, op, p, m, n, k) in warm]
    srv.replay(wreq, [0.0] * len(wreq))
    srv.drain()
    srv.close()
    torch.cuda.synchronize()

    srv = serve.Server(workers=W, hbm_budget=W * reserve, scratch_reserve=reserve)
    clocks = Clocks(0)
    clocks.start()
    time.sleep(0.25)
    t0 = srv.replay(reqs, offsets)
    srv.drain()
    clk = clocks.stop()
    st = srv.stats()
    bst = srv.batch_stats()
    srv.close()
    span = st["completed"] / st["solves_per_s"] if st["solves_per_s"] > 0 else float("nan")
    flops = sum(w[0] for w in work)

    # per-call baselines on a sample of the same stream
    vp = C.c_void_p

    def call(r):
        p, o = r.precision, r.op
        f, fl = (r.flags[0], r.flags[1], r.flags[2]), None
        if o == serve.GEMM:
            fn = L.exo_sgemm if p == 1 else L.exo_dgemm
            fn(101, f[0], f[1], r.m, r.n, r.k, r.alpha, vp(r.A), r.lda, vp(r.B), r.ldb, r.beta, vp(r.C), r.ldc)
        elif o == serve.SYRK:
            fn = L.exo_ssyrk if p == 1 else L.exo_dsyrk
            fn(101, f[0], f[1], r.m, r.k, r.alpha, vp(r.A), r.lda, r.beta, vp(r.C), r.ldc)
        elif o == serve.GEMV:
            fn = L.exo_sgemv if p == 1 else L.exo_dgemv
            fn(101, f[0], r.m, r.n, r.alpha, vp(r.A), r.lda, vp(r.B), r.ldb, r.beta, vp(r.C), r.ldc)
        else:
            fn = L.exo_strsv if p == 1 else L.exo_dtrsv
            fn(101, f[0], f[1], f[2], r.m, vp(r.A), r.lda, vp(r.C), r.ldc)
        st_ = L.exoblas_get_status()
        if st_:
            raise RuntimeError(f"per-call request failed with status {st_}")

    sample = reqs[:max(1, min(args.per_call_sample, len(reqs)))]

    def per_call(same_paths):
        eb.set_stream(None)
        eb.set_blocking(True)
        lat = []
        for r in sample[:50]:  # warm
            eb.set_precision(0 if not same_paths else (1 if r.precision == 1 else 2))
            call(r)
        t = time.perf_counter()
        for r in sample:
            if same_paths:
                eb.set_precision(1 if r.precision == 1 else 2)
            else:
                eb.set_precision(0)
            a = time.perf_counter()
            call(r)
            lat.append(time.perf_counter() - a)
        tot = time.perf_counter() - t
        eb.set_precision(0)
        eb.set_blocking(False)
        lat.sort()
        return {"solves_per_s": round(len(sample) / tot, 1), "seconds": round(tot, 3),
                "service_p50_ms": round(lat[len(lat) // 2] * 1e3, 3),
                "service_p99_ms": round(lat[min(len(lat) - 1, int(0.99 * (len(lat) - 1) + 0.5))] * 1e3, 3)}

    base = per_call(False)
    same = per_call(True)
    # the server on exactly the per-call sample (same requests, same arrival
    # offsets), so the ratios below compare one request set
    srv = serve.Server(workers=W, hbm_budget=W * reserve, scratch_reserve=reserve)
    srv.replay(sample, offsets[:len(sample)])
    srv.drain()
    st_s = srv.stats()
    srv.close()
    err = serve_errors(torch, eb, call, stream, built)
    line = {
        "metric": METRIC, "unit": "solves/s", "value": round(st["solves_per_s"], 1), "higher_is_better": True,
        "n_gpus": 1, "dtype": "f32 (split-BF16) + f64 (Ozaki)", "data": "synthetic",
        "config": {"workload": f"serve: Poisson {args.rate:g} req/s (seed 11), gemm 60%/gemv 25%/trsv 10%/syrk 5%, "
                               "m,n,k log-uniform [32,8192], 70% fp32 / 30% fp64 (seed 12), operands resident",
                   "requests": len(reqs), "workers": W, "admission_budget_gb": round(W * reserve / 1e9, 1)},
        "completed": int(st["completed"]), "rejected": int(st["rejected"]), "failed": int(st["failed"]),
        "p50_ms": round(st["p50_s"] * 1e3, 3), "p99_ms": round(st["p99_s"] * 1e3, 3),
        "mean_ms": round(st["mean_s"] * 1e3, 3), "max_ms": round(st["max_s"] * 1e3, 3),
        "span_s": round(span, 3), "arrival_span_s": round(offsets[-1], 3),
        "effective_tflops": round(flops / span / 1e12, 2) if span == span else None,
        "per_call_native": dict(base, sample=len(sample)),
        "per_call_same_paths": dict(same, sample=len(sample)),
        "device_batches": {"requests": bst["batched"], "batches": bst["batches"],
                           "requests_per_batch": round(bst["per_batch"], 1)},
        "server_on_sample": {"solves_per_s": round(st_s["solves_per_s"], 1), "p50_ms": round(st_s["p50_s"] * 1e3, 3),
                             "p99_ms": round(st_s["p99_s"] * 1e3, 3), "sample": len(sample)},
        "speedup_vs_per_call": round(st_s["solves_per_s"] / base["solves_per_s"], 2),
        "speedup_vs_per_call_same_paths": round(st_s["solves_per_s"] / same["solves_per_s"], 2),
        "error": err, "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def serve_errors(torch, eb, call, stream, built, per_kind=12, max_work=1 << 30):
    """Componentwise error max |r - e| / (|alpha||A||B| + |beta||C|) of the
    served paths (split-BF16, Ozaki) and of the native per-call kernels on
    gemm requests of the stream (m n k <= max_work), against torch FP64
    (FP32 requests) or against each other (FP64 requests)."""
    out = {"fp32_split_max": 0.0, "fp32_native_max": 0.0, "fp64_ozaki_vs_native_max": 0.0, "checked": 0}
    seen = {1: 0, 2: 0}
    eb.set_blocking(True)
    for (_, op, p, m, n, k), (r, views) in zip(stream, built):
        if op != "gemm" or m * n * k > max_work or seen[p] >= per_kind:
            continue
        seen[p] += 1
        A, B, Cm = views
        C0 = Cm.clone()
        A2, B2 = A.view(m, k).double(), B.view(k, n).double()
        mag = (A2.abs() @ B2.abs()) * abs(r.alpha) + C0.view(m, n).double().abs() * abs(r.beta)
        res = {}
        for mode in (0, 1 if p == 1 else 2):
            Cm.copy_(C0)
            torch.cuda.synchronize()
            eb.set_precision(mode)
            call(r)
            res[mode] = Cm.view(m, n).double().clone()
        eb.set_precision(0)
        Cm.copy_(C0)
        torch.cuda.synchronize()
        if p == 1:
            ref = r.alpha * (A2 @ B2) + r.beta * C0.view(m, n).double()
            out["fp32_native_max"] = max(out["fp32_native_max"], float(((res[0] - ref).abs() / mag).max()))
            out["fp32_split_max"] = max(out["fp32_split_max"], float(((res[1] - ref).abs() / mag).max()))
        else:
            out["fp64_ozaki_vs_native_max"] = max(out["fp64_ozaki_vs_native_max"],
                                                  float(((res[2] - res[0]).abs() / mag).max()))
        out["checked"] += 1
    eb.set_blocking(False)
    return {k: (float(f"{v:.3e}") if isinstance(v, float) else v) for k, v in out.items()}


def run_reference(args):
    """The reference's CPU path (the oracle's restatement of the Exo
    algorithms, threaded over ranges / rows) on all host cores, over the full
    bandwidth set: warm-up of max(--warmup passes, 1 s), then max(--steps
    passes, 1 s) timed; value = the median pass."""
    threads = cpu_threads()
    S = cpu_inputs()
    m = cpu_measure(S, threads, warm_passes=args.warmup, passes=args.steps)
    v = m["value"]
    cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": CPU_DESC,
           "protocol": CPU_PROTOCOL, "passes": m["passes"], "seconds": m["seconds"], "spread": m["spread"]}
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": m["passes"], "warmup": m["warmup_passes"], "ms_per_step": m["ms_per_pass"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "impl": "reference", "config": {"workload": WORKLOAD, "sample": CPU_DESC, "same_config": True},
        "cpu_baseline": cpu,
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
