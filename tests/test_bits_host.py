"""The integer float <-> double conversions the node update uses on the
device (openradioss_gb300/csrc/rg_bits.h: widen_f32, narrow_f64 and the node
code extraction small_int_f64) return exactly what the IEEE conversions
return: the header compiled as host C++ against the host's own conversions,
over a stride of every float bit pattern, 20 million random doubles, the
rounding boundaries (dropped bits at and next to one half) across the float
exponent range and the edge values (zeros, subnormals, overflow, inf, NaN)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_bit_conversions_match_ieee(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "bits_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-o", exe,
                    os.path.join(HERE, "native", "bits_check.cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    bad, n = (int(x) for x in r.stdout.split()[-2:])
    assert r.returncode == 0 and bad == 0, r.stdout
    assert n > 100_000_000
