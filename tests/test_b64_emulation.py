"""The integer binary64 primitives (rebop_gb300/csrc/b64.cuh) equal the host FPU bit for bit.

The kernels use these primitives in place of binary64 instructions; the same
header compiles for the host, where tests/b64_check.cpp compares each
operation against IEEE round-to-nearest-even hardware results.
"""

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("n", [600_000])
def test_b64_primitives_match_host_fpu(tmp_path, n):
    exe = tmp_path / "b64_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(ROOT / "rebop_gb300" / "csrc"),
                    str(ROOT / "tests" / "b64_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(n)], check=True, capture_output=True, text=True).stdout
    rows = {line.split()[0]: [int(x) for x in line.split()[1:]] for line in out.strip().splitlines()}
    assert set(rows) == {"from_u53", "mul_int", "mul_u32", "mul_u64", "add", "sub", "div", "div_exact"}
    for op, (cases, mismatches, refused) in rows.items():
        assert cases > 0 and mismatches == 0, f"{op}: {mismatches} mismatches in {cases}"
        assert refused < cases // 20, f"{op}: refused {refused} of {cases}"
