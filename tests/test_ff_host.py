"""The mixed form's double-float arithmetic and FP32 contact law checked on the CPU.

`gorilla-physics_gb300/csrc/gpb_ff.cuh` and the double-float 6×6 factor and
solve of a floating joint (`chol6_ff`, `solve6_ff` in `gpb_aba.cuh`) are
compiled as plain C++ from the kernel sources themselves, with host versions of
the round-to-nearest intrinsics they call (`__fadd_rn`, `__fmul_rn`,
`__fmaf_rn`, ...; contraction off, so each is one correctly rounded FP32
operation) and an `rsqrtf` perturbed by up to 2 ulp either way (the device one
is approximate).  `tests/ff_host_check.cpp` checks them against long double:
two_sum exact; ff_add commutative bit for bit; ff_add, ff_mul, ff_fma, ff_rcp
within 3e-14; ff_rsqrt within 3e-13 (one Newton step leaves 1.5·δ² of a start
off by δ: 2.6e-14 from a correctly rounded FP32 start, 1.9e-13 from one 2 ulp
off); the 6×6 factor of 20,000 random spatial inertias (rigid bodies plus
random articulated parts) with its reciprocal pivots within 1e-12 and its
solve within 1e-10 of max|x|; an indefinite matrix reported.

The contact law the mixed form runs in FP32 (`contact_force_parts` in
`gpb_kernels.cu`, fed with the approach speed and tangential velocity formed in
FP64) is compiled the same way and compared with the FP64 form's
`contact_force<double>` on 800,000 contact states of both laws: stiffnesses of
the cube and quadruped configurations, penetrations inside the 1e-8 margin to
5 cm, tangential speeds from 1 down to 1e-9 through the 1e-3 friction
regularisation.  The force error stays within 1e-6 of the size of the terms
the law adds ((|k z| + |c ż|)(1 + μ); Hunt–Crossley alike), and the FP64 form's
law is the same arithmetic as its parts form, bit for bit.
"""

import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "gorilla-physics_gb300" / "csrc"

HOST = r"""
#include <cmath>
#define __device__
#define __forceinline__ inline
static inline float __fadd_rn(float a, float b) { volatile float r = a + b; return r; }
static inline float __fsub_rn(float a, float b) { volatile float r = a - b; return r; }
static inline float __fmul_rn(float a, float b) { volatile float r = a * b; return r; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
static inline float __frcp_rn(float a) { volatile float r = 1.0f / a; return r; }
static inline float __double2float_rn(double x) { return (float)x; }
float rsqrtf_host(float x);
#define rsqrtf rsqrtf_host
"""


def _between(text, start, end):
    i = text.index(start)
    return text[i:text.index(end, i)]


def harness_header() -> str:
    ff = (CSRC / "gpb_ff.cuh").read_text().replace("#pragma once", "")
    aba = (CSRC / "gpb_aba.cuh").read_text()
    abif = re.search(r"struct ABIF \{[^}]*\};", aba).group(0)
    symget = _between(aba, "template <typename T>\n__device__ __forceinline__ T symget", "\ntemplate") + "\n"
    l6 = re.search(r"__device__ __forceinline__ int l6\(int i, int j\) \{[^}]*\}", aba).group(0)
    chol = _between(aba, "__device__ __forceinline__ bool chol6_ff", "// Per-DOF record of the inward pass")
    return HOST + ff + abif + "\n" + symget + l6 + "\n" + chol


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs a host C++ compiler")
def test_double_float_arithmetic_on_host(tmp_path):
    (tmp_path / "ff_harness.h").write_text(harness_header())
    exe = tmp_path / "ff_host_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(tmp_path),
                    str(ROOT / "tests" / "ff_host_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    out = dict(line.split() for line in r.stdout.splitlines() if not line.startswith("FAIL"))
    assert r.returncode == 0, r.stdout
    assert float(out["solve6_ff_rel_err"]) <= 1e-10
    assert float(out["chol6_ff_indefinite_missed"]) == 0


LAW_HOST = r"""
#include <cmath>
#define __device__
#define __forceinline__ inline
namespace gpb {
using std::fmax;
using std::sqrt;
"""


def law_header() -> str:
    dev = (CSRC / "gpb_device.cuh").read_text()
    vec = _between(dev, "template <typename R>\nstruct V3", "// Row-major 3x3.")
    ker = (CSRC / "gpb_kernels.cu").read_text()
    law = _between(ker, "// Contact force of one point against one half-space",
                   "// ---------------------------------------------------------------------------\n// Cuboid colliders")
    return LAW_HOST + vec + law + "}  // namespace gpb\n"


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs a host C++ compiler")
def test_mixed_contact_law_on_host(tmp_path):
    (tmp_path / "law_harness.h").write_text(law_header())
    exe = tmp_path / "contact_law_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(tmp_path),
                    str(ROOT / "tests" / "contact_law_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    out = dict(line.split() for line in r.stdout.splitlines())
    assert float(out["fp64_parts_differ"]) == 0
