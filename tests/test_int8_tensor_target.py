"""Why the Ozaki dgemm carries its slices as BF16 digits, not INT8: sm_103a
(GB300) has no integer tcgen05 MMA.  ptxas rejects `tcgen05.mma ...
.kind::i8` for sm_103a and accepts the same instruction for sm_100a, while
`.kind::f16` (BF16 / FP16 operands) assembles for both.  Compile-only: no
GPU is used."""
import shutil
import subprocess

import pytest

_SRC = r"""
#include <cstdint>
__global__ void k(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, int acc) {
  asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
               "tcgen05.mma.cta_group::1.kind::KIND [%0], %1, %2, %3, p;\n}\n"
               :: "r"(tmem), "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
"""


def _compile(tmp_path, kind, arch):
    src = tmp_path / f"mma_{kind}_{arch}.cu"
    src.write_text(_SRC.replace("KIND", kind))
    r = subprocess.run(["nvcc", "-gencode", f"arch=compute_{arch},code=sm_{arch}", "-c", str(src), "-o",
                        str(tmp_path / f"{src.stem}.o")], capture_output=True, text=True)
    return r.returncode, r.stderr


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not found")
def test_int8_mma_is_not_available_on_sm_103a(tmp_path):
    rc, err = _compile(tmp_path, "i8", "103a")
    assert rc != 0 and "not supported on .target 'sm_103a'" in err
    assert _compile(tmp_path, "i8", "100a")[0] == 0
    assert _compile(tmp_path, "f16", "103a")[0] == 0
