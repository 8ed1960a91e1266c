"""The integer-pipe FP64 operations (mycode_gb300/csrc/exact64.cuh: x / 2, 2 x and the
comparisons the bit-exact residual takes off the FP64 pipe) against the FP64 instructions,
bit for bit, on random doubles of every magnitude and on the special values: signed zeros,
subnormals (both ends, and the halving ties), the smallest normals, the largest finite
values, infinities.  Comparisons are checked on non-NaN operands."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _values():
    rng = np.random.default_rng(11)
    tiny = np.finfo(np.float64).tiny
    sub = np.array([5e-324, 1e-323, 1.5e-323, 2e-323, tiny / 2, tiny - 5e-324, tiny, tiny + 5e-324, 2 * tiny,
                    np.finfo(np.float64).max, np.finfo(np.float64).max / 2, 8.98846567431158e307, 0.0, 1.0, 0.5, 2.0])
    bits = rng.integers(0, 2**63 - 2**52, size=20000, dtype=np.int64)  # every finite exponent
    rnd = bits.view(np.float64)
    subs = rng.integers(1, 2**52, size=4000, dtype=np.int64).view(np.float64)  # subnormals
    v = np.concatenate([sub, -sub, [np.inf, -np.inf, -0.0], rnd, -rnd, subs, -subs,
                        rng.standard_normal(4000) * 1e5])
    return v[np.isfinite(v) | np.isinf(v)]


def test_exact64_ops_equal_fp64_instructions(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = tmp_path / "exact64_check"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-o", str(exe),
                    os.path.join(HERE, "exact64", "exact64_check.cu")], check=True)
    v = _values()
    (tmp_path / "in.bin").write_bytes(v.tobytes())
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    o = np.frombuffer((tmp_path / "out.bin").read_bytes(), dtype=np.uint64).reshape(-1, 10)
    assert o.shape[0] == v.size
    np.testing.assert_array_equal(o[:, 0], o[:, 1])  # x / 2
    np.testing.assert_array_equal(o[:, 2], o[:, 3])  # 2 x
    np.testing.assert_array_equal(o[:, 4], o[:, 5])  # a < b
    np.testing.assert_array_equal(o[:, 6], o[:, 7])  # x > 0
    np.testing.assert_array_equal(o[:, 8], o[:, 9])  # x < 0
    # the numpy FP64 results too (host IEEE arithmetic; 2 x of the largest binade overflows)
    with np.errstate(over="ignore"):
        np.testing.assert_array_equal(o[:, 0], (v * 0.5).view(np.uint64))
        np.testing.assert_array_equal(o[:, 2], (v * 2.0).view(np.uint64))


def test_tanh_saturation_equals_cuda_tanh(tmp_path):
    """The SST model's tanh_sat (1 from 19.5 in FP64 / 9.5 in FP32 on, x below 2^-27 /
    2^-13) against CUDA's tanh and tanhf bit for bit: dense samples on both sides of both
    thresholds, every exponent above and below them, and the special values."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = tmp_path / "tanh_check"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-o", str(exe),
                    os.path.join(HERE, "exact64", "tanh_check.cu")], check=True)
    rng = np.random.default_rng(5)
    v = np.concatenate([
        np.linspace(0.0, 30.0, 600001),                 # through both upper thresholds
        rng.uniform(8.0, 25.0, 400000),
        np.exp(rng.uniform(np.log(25.0), np.log(1e300), 100000)),
        np.exp(rng.uniform(np.log(1e-320), np.log(1e-2), 400000)),  # through both lower thresholds
        [0.0, -0.0, 5e-324, np.inf, 2.0 ** -27, np.nextafter(2.0 ** -27, 0), 2.0 ** -13, 19.5, 9.5],
    ])
    v = np.concatenate([v, -v[: 200000]])
    (tmp_path / "in.bin").write_bytes(v.astype(np.float64).tobytes())
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    o = np.frombuffer((tmp_path / "out.bin").read_bytes(), dtype=np.uint64).reshape(-1, 4)
    assert o.shape[0] == v.size
    bad64 = np.nonzero(o[:, 0] != o[:, 1])[0]
    bad32 = np.nonzero(o[:, 2] != o[:, 3])[0]
    assert bad64.size == 0, v[bad64[:5]]
    assert bad32.size == 0, v[bad32[:5]]
