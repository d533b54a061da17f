// sg_healpix.h -- HEALPix helpers used to choose the library's internal
// pixel numbering (plain C++; the integer ring -> nested map also compiles
// for the device).
//
// The reference numbers observed pixels in ascending RING order (indpix,
// sanepic.cc:904-915).  Internally the library numbers them in NESTED order
// instead: NESTED indices follow a quadtree over the 12 base faces, so pixels
// that are close on the sky are close in the index.  Two things depend on
// that: P^T gathers samples pixel by pixel, and neighbouring pixels along the
// scan then share cache lines; and nested blocks of 4^k consecutive pixels are
// the compact patches the learned preconditioner works on.  Maps are converted
// back to RING order at the API boundary.
//
// Restated from the HEALPix pixelisation (Gorski et al. 2005, ApJ 622, 759):
// ring pixel centres (z = cos theta, phi), and the nested index of a
// direction from its base face and the (x, y) position inside the face.
#pragma once
#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define SG_HD __host__ __device__
#else
#define SG_HD
#endif

namespace sg {

inline long long hp_isqrt(long long v) {
  long long r = (long long)std::sqrt((double)v);
  while (r * r > v) r--;
  while ((r + 1) * (r + 1) <= v) r++;
  return r;
}

// centre of RING pixel p: z = cos(theta), phi in [0, 2 pi)
inline void hp_pix2ang_ring(long long nside, long long p, double* z, double* phi) {
  const double pi = 3.14159265358979323846;
  const long long ncap = 2 * nside * (nside - 1), npix = 12 * nside * nside;
  const double fact2 = 4.0 / (double)npix;  // 1 / (3 nside^2)
  if (p < ncap) {
    const long long iring = (1 + hp_isqrt(1 + 2 * p)) >> 1;
    const long long iphi = p + 1 - 2 * iring * (iring - 1);
    *z = 1.0 - (double)(iring * iring) * fact2;
    *phi = ((double)iphi - 0.5) * pi / (2.0 * (double)iring);
  } else if (p < npix - ncap) {
    const long long ip = p - ncap;
    const long long iring = ip / (4 * nside) + nside;
    const long long iphi = ip % (4 * nside) + 1;
    const double fodd = ((iring + nside) & 1) ? 1.0 : 0.5;
    *z = (double)(2 * nside - iring) * 2.0 / (3.0 * (double)nside);
    *phi = ((double)iphi - fodd) * pi / (2.0 * (double)nside);
  } else {
    const long long ip = npix - p;
    const long long iring = (1 + hp_isqrt(2 * ip - 1)) >> 1;
    const long long iphi = 4 * iring + 1 - (ip - 2 * iring * (iring - 1));
    *z = -1.0 + (double)(iring * iring) * fact2;
    *phi = ((double)iphi - 0.5) * pi / (2.0 * (double)iring);
  }
}

// spread the low 32 bits of v to the even bit positions
inline uint64_t hp_spread(uint64_t v) {
  v &= 0xffffffffULL;
  v = (v | (v << 16)) & 0x0000ffff0000ffffULL;
  v = (v | (v << 8)) & 0x00ff00ff00ff00ffULL;
  v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0fULL;
  v = (v | (v << 2)) & 0x3333333333333333ULL;
  v = (v | (v << 1)) & 0x5555555555555555ULL;
  return v;
}

// NESTED index of direction (z, phi); nside must be a power of two
inline long long hp_ang2pix_nest(long long nside, double z, double phi) {
  const double pi = 3.14159265358979323846;
  const double za = std::fabs(z);
  double tt = std::fmod(phi, 2.0 * pi);
  if (tt < 0.0) tt += 2.0 * pi;
  tt /= 0.5 * pi;  // in [0, 4)
  long long face, ix, iy;
  if (za <= 2.0 / 3.0) {
    const double t1 = (double)nside * (0.5 + tt);
    const double t2 = (double)nside * z * 0.75;
    const long long jp = (long long)(t1 - t2);  // ascending edge line
    const long long jm = (long long)(t1 + t2);  // descending edge line
    const long long ifp = jp / nside, ifm = jm / nside;
    face = (ifp == ifm) ? (ifp | 4) : ((ifp < ifm) ? ifp : ifm + 8);
    ix = jm & (nside - 1);
    iy = nside - (jp & (nside - 1)) - 1;
  } else {
    long long ntt = (long long)tt;
    if (ntt >= 4) ntt = 3;
    const double tp = tt - (double)ntt;
    const double tmp = (double)nside * std::sqrt(3.0 * (1.0 - za));
    long long jp = (long long)(tp * tmp), jm = (long long)((1.0 - tp) * tmp);
    if (jp > nside - 1) jp = nside - 1;
    if (jm > nside - 1) jm = nside - 1;
    if (z >= 0.0) {
      face = ntt;
      ix = nside - jm - 1;
      iy = nside - jp - 1;
    } else {
      face = ntt + 8;
      ix = jp;
      iy = jm;
    }
  }
  return face * nside * nside + (long long)(hp_spread((uint64_t)ix) | (hp_spread((uint64_t)iy) << 1));
}

// NESTED index of RING pixel p (via its centre)
inline long long hp_ring2nest(long long nside, long long p) {
  double z, phi;
  hp_pix2ang_ring(nside, p, &z, &phi);
  return hp_ang2pix_nest(nside, z, phi);
}

// The same map in integer arithmetic only (host and device): the ring number
// and in-ring index of p give the pixel centre's face coordinates exactly.
// Equatorial rings (nside <= i <= 3 nside): with f2 = 2 if i + nside is odd
// (the ring's first centre sits at phi = pi / (2 nside)) else 1, the centre's
// coordinates along the ascending and descending face edges are the
// half-integers (2 iphi - f2 + i - nside) / 2 and (2 iphi - f2 + 3 nside - i) / 2.
// Polar rings (i < nside from either pole) hold i pixels per face; the k-th
// face's p-th pixel (1-based) sits at edge coordinates (p - 1/2, i - p + 1/2).
SG_HD inline long long hp_isqrt_int(long long v) {
  long long r = 0, b = 1LL << 62;
  while (b > v) b >>= 2;
  while (b != 0) {
    if (v >= r + b) {
      v -= r + b;
      r = (r >> 1) + b;
    } else {
      r >>= 1;
    }
    b >>= 2;
  }
  return r;
}

SG_HD inline uint64_t hp_spread_int(uint64_t v) {
  v &= 0xffffffffULL;
  v = (v | (v << 16)) & 0x0000ffff0000ffffULL;
  v = (v | (v << 8)) & 0x00ff00ff00ff00ffULL;
  v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0fULL;
  v = (v | (v << 2)) & 0x3333333333333333ULL;
  v = (v | (v << 1)) & 0x5555555555555555ULL;
  return v;
}

SG_HD inline long long hp_ring2nest_int(long long nside, long long p) {
  const long long ncap = 2 * nside * (nside - 1), npix = 12 * nside * nside;
  long long face, ix, iy;
  if (p >= ncap && p < npix - ncap) {
    const long long ip = p - ncap;
    const long long i = ip / (4 * nside) + nside;
    const long long iphi = ip % (4 * nside) + 1;
    const long long f2 = ((i + nside) & 1) ? 2 : 1;
    const long long jp = (2 * iphi - f2 + i - nside - 1) / 2;
    const long long jm = (2 * iphi - f2 + 3 * nside - i - 1) / 2;
    const long long ifp = jp / nside, ifm = jm / nside;
    face = (ifp == ifm) ? (ifp | 4) : ((ifp < ifm) ? ifp : ifm + 8);
    ix = jm & (nside - 1);
    iy = nside - (jp & (nside - 1)) - 1;
  } else {
    const bool north = p < ncap;
    const long long ip = north ? p + 1 : npix - p;  // 1-based from the pole
    const long long i = north ? (1 + hp_isqrt_int(2 * ip - 1)) >> 1
                              : (1 + hp_isqrt_int(2 * ip - 1)) >> 1;
    const long long iphi = north ? ip - 2 * i * (i - 1) : 4 * i + 1 - (ip - 2 * i * (i - 1));
    const long long k = (iphi - 1) / i, q = iphi - k * i;
    const long long jp = q - 1, jm = i - q;
    if (north) {
      face = k;
      ix = nside - jm - 1;
      iy = nside - jp - 1;
    } else {
      face = k + 8;
      ix = jp;
      iy = jm;
    }
  }
  return face * nside * nside +
         (long long)(hp_spread_int((uint64_t)ix) | (hp_spread_int((uint64_t)iy) << 1));
}

}  // namespace sg
