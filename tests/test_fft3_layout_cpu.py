"""Host logic of the three-pass FP32 weighting (sanepic_gb300/csrc/sg_fft3.cu),
no GPU: the position order of its spectra and weights is a permutation of the
M + 1 frequencies, every frequency k = k1 + R k2 sits at position C k1 + k2
with its real-FFT partner M - k in row R - k1 (row 0: itself) as the row
kernels assume, and the single-timeline batches fit the L2 budget."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "sanepic_gb300", "csrc")
SRC = r"""
#include "sg_fft3.cu"
extern "C" int t_pos_freq(int logm, int* out) {
  std::vector<int> k;
  sg::fft3_pos_freq(logm, k);
  for (size_t i = 0; i < k.size(); i++) out[i] = k[i];
  return (int)k.size();
}
extern "C" long long t_batch(int logm) { return sg::fft3_rhs_batch(logm); }
extern "C" int t_supported(int logm) { return sg::fft3_supported(logm) ? 1 : 0; }
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    d = tmp_path_factory.mktemp("f3")
    (d / "t.cu").write_text(SRC)
    so = d / "t.so"
    subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O1", "-std=c++17",
                           "-shared", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                           "-I", CSRC, "-I", os.path.join(ROOT, "include"), str(d / "t.cu"),
                           "-o", str(so)])
    L = ctypes.CDLL(str(so))
    L.t_pos_freq.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.t_batch.restype = ctypes.c_longlong
    return L


@pytest.mark.parametrize("logm", range(10, 17))
def test_positions_are_a_permutation_with_partners_in_paired_rows(lib, logm):
    assert lib.t_supported(logm) == 1
    M = 1 << logm
    R = 1 << (logm // 2)
    C = M // R
    k = np.zeros(M + 1, np.int32)
    assert lib.t_pos_freq(logm, k.ctypes.data_as(ctypes.POINTER(ctypes.c_int))) == M + 1
    assert np.array_equal(np.sort(k), np.arange(M + 1))
    pos = np.empty(M + 1, np.int64)
    pos[k] = np.arange(M + 1)
    kk = np.arange(1, M)
    p, q = pos[kk], pos[M - kk]
    k1, k2 = p // C, p % C
    pk1, pk2 = q // C, q % C
    # rows k1 and R - k1 (mod R) pair up; columns as the row kernels' tasks
    assert np.array_equal(pk1, (R - k1) % R)
    inner = k1 != 0
    assert np.array_equal(pk2[inner], C - 1 - k2[inner])
    assert np.array_equal(pk2[~inner], (C - k2[~inner]) % C)
    assert pos[0] == 0 and pos[M] == M


@pytest.mark.parametrize("logm", [10, 13, 16])
def test_batches_fit_the_l2_budget(lib, logm):
    nb = lib.t_batch(logm)
    assert nb >= 1 and nb * (8 << logm) <= 48 << 20
    assert lib.t_supported(9) == 0 and lib.t_supported(17) == 0
