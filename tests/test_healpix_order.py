"""The library's internal NESTED pixel numbering (sanepic_gb300/csrc/sg_healpix.h):
ring pixel centres map back to themselves through the reference's ang2pix_ring
(restated in the oracle), the nested indices are a permutation, and blocks of
256 consecutive nested indices are compact sky patches."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = """
#include "sg_healpix.h"
extern "C" long long t_ring2nest(long long nside, long long p) { return sg::hp_ring2nest(nside, p); }
extern "C" void t_pix2ang(long long nside, long long p, double* z, double* phi) {
  sg::hp_pix2ang_ring(nside, p, z, phi);
}
// pixels where the integer map differs from the map through the pixel centre
extern "C" long long t_int_mismatches(long long nside) {
  long long bad = 0;
  for (long long p = 0; p < 12 * nside * nside; p++)
    bad += sg::hp_ring2nest_int(nside, p) != sg::hp_ring2nest(nside, p);
  return bad;
}
"""


@pytest.fixture(scope="module")
def hp(tmp_path_factory):
    d = tmp_path_factory.mktemp("hp")
    src = d / "hp.cpp"
    src.write_text(SRC)
    so = d / "hp.so"
    subprocess.check_call(["g++", "-O2", "-shared", "-fPIC", "-I",
                           os.path.join(ROOT, "sanepic_gb300", "csrc"), str(src), "-o", str(so)])
    L = ctypes.CDLL(str(so))
    L.t_ring2nest.restype = ctypes.c_longlong
    L.t_ring2nest.argtypes = [ctypes.c_longlong, ctypes.c_longlong]
    L.t_int_mismatches.restype = ctypes.c_longlong
    L.t_int_mismatches.argtypes = [ctypes.c_longlong]
    L.t_pix2ang.argtypes = [ctypes.c_longlong, ctypes.c_longlong,
                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    return L


def centres(L, nside):
    npix = 12 * nside * nside
    z, phi = np.empty(npix), np.empty(npix)
    zz, pp = ctypes.c_double(), ctypes.c_double()
    for p in range(npix):
        L.t_pix2ang(nside, p, ctypes.byref(zz), ctypes.byref(pp))
        z[p], phi[p] = zz.value, pp.value
    return z, phi


@pytest.mark.parametrize("nside", [1, 2, 4, 8, 16])
def test_centres_round_trip_through_reference_ang2pix(hp, nside):
    z, phi = centres(hp, nside)
    back = oracle.ang2pix_ring(nside, np.arccos(z), phi)
    assert np.array_equal(back, np.arange(12 * nside * nside))


@pytest.mark.parametrize("nside", [1, 2, 4, 8, 16, 32])
def test_nested_is_a_permutation(hp, nside):
    npix = 12 * nside * nside
    nest = np.array([hp.t_ring2nest(nside, p) for p in range(npix)])
    assert np.array_equal(np.sort(nest), np.arange(npix))


def test_nested_blocks_are_compact(hp):
    nside = 64
    npix = 12 * nside * nside
    z, phi = centres(hp, nside)
    nest = np.array([hp.t_ring2nest(nside, p) for p in range(npix)])
    order = np.argsort(nest)
    th = np.arccos(z)
    v = np.stack([np.sin(th) * np.cos(phi), np.sin(th) * np.sin(phi), z], 1)[order]
    worst = 0.0
    for b in range(0, npix, 256):
        blk = v[b:b + 256]
        c = blk.mean(0)
        c /= np.linalg.norm(c)
        worst = max(worst, np.degrees(np.arccos(np.clip(blk @ c, -1, 1))).max())
    # a 16 x 16 nested block at nside 64 is ~15 deg across
    assert worst < 15.0


@pytest.mark.parametrize("nside", [1, 2, 4, 8, 16, 32, 64, 128, 256, 512])
def test_integer_ring2nest_matches_centre_map(hp, nside):
    """the integer map the library runs on the GPU equals the map through
    the pixel centres, pixel for pixel"""
    assert hp.t_int_mismatches(nside) == 0
