"""Non-blocking mode (exoblas_set_blocking(0)): calls on device operands
return after queuing their kernels on the thread's stream, reductions write
device results, and exoblas_synchronize() completes the queue.  A dependent
pipeline run that way must give the blocking results."""
import numpy as np
import pytest


@pytest.mark.gpu
def test_nonblocking_device_pipeline(cuda):
    import torch

    import exoblas_gb300 as eb

    g = torch.Generator(device="cuda").manual_seed(9)
    n, m = 1 << 20, 1536
    x = torch.rand(n, generator=g, device="cuda") * 2 - 1
    y = torch.rand(n, generator=g, device="cuda") * 2 - 1
    A = (torch.rand((m, m), generator=g, device="cuda") * 2 - 1).contiguous()
    L = torch.tril(torch.rand((m, m), generator=g, device="cuda") / m)
    L.diagonal().copy_(1 + torch.rand(m, generator=g, device="cuda"))
    v = torch.rand(m, generator=g, device="cuda") * 2 - 1
    x64, y64, A64, L64, v64 = x.double(), y.double(), A.double(), L.double(), v.double()
    torch.cuda.synchronize()

    res = torch.zeros(2, dtype=torch.float32, device="cuda")
    w = torch.zeros(m, dtype=torch.float32, device="cuda")
    eb.set_blocking(False)
    try:
        eb.exo_saxpy(n, 0.5, x, 1, y, 1)                          # y <- y + x/2
        eb.exoblas_sdot_device(n, x, 1, y, 1, res[0:1])            # uses the new y
        eb.exo_sgemv(101, 111, m, m, 1.0, A, m, v, 1, 0.0, w, 1)  # w <- A v
        eb.exo_strsv(101, 122, 111, 131, m, L, m, w, 1)           # w <- L^-1 w
        eb.exoblas_sasum_device(m, w, 1, res[1:2])                 # uses the solved w
        eb.synchronize()
    finally:
        eb.set_blocking(True)

    y_ref = y64 + 0.5 * x64
    assert torch.allclose(y.double(), y_ref, rtol=0, atol=1e-6)
    dot_ref = float(x64 @ y_ref)
    assert abs(float(res[0]) - dot_ref) <= 4 * n * 1.2e-7 * float(x64.abs() @ y_ref.abs())
    w_ref = torch.linalg.solve_triangular(L64, (A64 @ v64).unsqueeze(1), upper=False).squeeze(1)
    resid = L64 @ w.double() - A64 @ v64
    assert float(resid.abs().max()) <= 8 * m * 1.2e-7 * float((L64.abs() @ w.double().abs()).max())
    assert abs(float(res[1]) - float(w.double().abs().sum())) <= 4 * m * 1.2e-7 * float(w.double().abs().sum())
    assert float((w.double() - w_ref).abs().max()) <= 1e-3
