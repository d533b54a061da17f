// sg_pointing.cu -- per-detector pointing expansion and HEALPix RING
// pixelisation on the GPU, in FP64.
//
// Restates, per sample, the reference's pointingshift (sanepic.cc:3412-3476),
// the detector-angle / HWP step (sanepic.cc:737-766) and ang2pix_ring
// (sanepic.cc:2764-2843, called at 855-874) with the same operation order.
// This translation unit is compiled with --fmad=false so that no a*b+c is
// contracted into an FMA: every +,-,*,/,sqrt,floor,fmod is the correctly
// rounded IEEE operation the reference performs.  The remaining difference
// from the host build is the last-bit accuracy of CUDA's FP64 sin/cos/acos/
// atan2/asin, which can move a pixel index only for a sample within ~1e-16
// of a pixel boundary.
//
// Detectors that share (offx, offy) have identical pixels and differ only by
// the constant angle psi[idet] added after pointingshift (the boresight files
// are common to all detectors, sanepic.cc:680-692, 757-766), so the kernel
// works per offset group: one RING pixel and one FP64 angle psi_o per group
// sample; the per-detector angle is applied later as a rotation.
#include <cuda_runtime.h>

#include "sg_kernels.h"

namespace sg {

#define SG_D2PI 6.2831853071795864769252867665590057683943387987502

__device__ __forceinline__ int ang2pix_ring_dev(long long nside, double theta, double phi) {
  int nl4, ncap, npix, jp, jm, ipix1;
  double z, za, tt, tp, tmp;
  int ir, ip, kshift;
  const double piover2 = 0.5 * 3.14159265358979323846;
  const double twopi = 2.0 * 3.14159265358979323846;
  const double z0 = 2.0 / 3.0;
  z = cos(theta);
  za = fabs(z);
  if (phi >= twopi) phi = phi - twopi;
  if (phi < 0.) phi = phi + twopi;
  tt = phi / piover2;
  nl4 = 4 * (int)nside;
  ncap = 2 * (int)nside * ((int)nside - 1);
  npix = 12 * (int)nside * (int)nside;
  const double dn = (double)nside;
  if (za <= z0) {
    jp = (int)floor(dn * (0.5 + tt - z * 0.75));
    jm = (int)floor(dn * (0.5 + tt + z * 0.75));
    ir = (int)nside + 1 + jp - jm;
    kshift = 0;
    if ((ir & 1) == 0) kshift = 1;
    // C integer division (truncation toward zero), as in the reference
    ip = (int)((long long)(jp + jm - (int)nside + kshift + 1) / 2) + 1;
    if (ip > nl4) ip = ip - nl4;
    ipix1 = ncap + nl4 * (ir - 1) + ip;
  } else {
    tp = tt - floor(tt);
    tmp = sqrt(3. * (1. - za));
    jp = (int)floor(dn * tp * tmp);
    jm = (int)floor(dn * (1. - tp) * tmp);
    ir = jp + jm + 1;
    ip = (int)floor(tt * ir) + 1;
    if (ip > 4 * ir) ip = ip - 4 * ir;
    ipix1 = 2 * ir * (ir - 1) + ip;
    if (z <= 0.) ipix1 = npix - 2 * ir * (ir + 1) + ip;
  }
  return ipix1 - 1;
}

__global__ void k_pointing(PointingArgs a) {
  const long long nsd = a.ns * a.nseg;
  const long long total = nsd * a.ngroups;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int g = (int)(e / nsd);
    const long long w = e % nsd;  // iseg * ns + ii
    const double x = a.offx[g], y = a.offy[g];
    // pointingshift with nn = 1 (sanepic.cc:3419-3471)
    const double thetap = SG_D2PI / 4.0 - a.dec[w];
    const double phip = a.ra[w];
    const double psip_b = a.psi[w];
    if (x == 0.0 && y == 0.0) {
      // Zero offset: theta_ = phi_ = 0 exactly, so every term carrying
      // sin(theta_) is a signed zero and adding it leaves the others
      // unchanged; what remains is the same operations on the same values:
      // theta_o = acos(cos thetap), phi_o = phip (atan2 of a signed zero over
      // sin thetap > 0), dr = (-cos thetap cos psi, -sin psi, sin thetap cos psi),
      // eph = (-0, 1, 0), so aaa = dr[1].  Poles and NaN angles take the
      // general path below.
      const double st = sin(thetap);
      if (st > 0.0 && psip_b == psip_b) {
        const double ct = cos(thetap), cp = cos(psip_b), sp = sin(psip_b);
        const double theta_o = acos(ct);
        const double phi_o = phip;
        const double dr0 = (-ct) * cp, dr1 = -sp, dr2 = st * cp;
        const double rrr = ((0.0 + dr0 * dr0) + dr1 * dr1) + dr2 * dr2;
        double aaa = dr1 / sqrt(rrr);
        if (aaa > 1.0) aaa = 1.0;
        if (aaa < -1.0) aaa = -1.0;
        double psitmp = acos(aaa);
        if (dr2 < 0) psitmp = -psitmp;
        const double psi_o =
            (fmod(psitmp + SG_D2PI / 4.0 + 2.0 * SG_D2PI, SG_D2PI)) - SG_D2PI / 2.0;
        const double theta = SG_D2PI / 4.0 - (SG_D2PI / 4.0 - theta_o);
        const double phi = fmod(phi_o + SG_D2PI, SG_D2PI);
        int pix;
        if (theta != theta || phi != phi) {
          pix = -1;
        } else if (theta < 0. || theta > 3.14159265358979323846) {
          pix = -2;
          atomicExch(a.error_flag, 1);
        } else {
          pix = ang2pix_ring_dev(a.nside, theta, phi);
          if (pix < 0 || pix > 12 * (int)a.nside * (int)a.nside - 1) pix = -1;
        }
        a.ring_pix[e] = pix;
        a.psio[e] = psi_o;
        continue;
      }
    }
    const double theta_ = asin(sqrt(x * x + y * y));
    const double phi_ = atan2(y, x);
    const double theta_o = acos(sin(thetap) * sin(theta_) * cos(phi_ + psip_b) +
                                cos(thetap) * cos(theta_));
    const double phi_o = atan2(-sin(theta_) * sin(phi_ + psip_b),
                               (-cos(thetap) * sin(theta_) * cos(phi_ + psip_b) +
                                sin(thetap) * cos(theta_))) +
                         phip;
    double drp[3], dr[3], eph[3], R[3][3];
    drp[2] = -sin(theta_) * cos(phi_);
    for (int i = 0; i < 3; i++)
      for (int k = 0; k < 3; k++) R[i][k] = 0.0;
    R[1][1] = -1.0;
    eph[2] = 0.0;
    drp[0] = cos(psip_b) * cos(theta_);
    drp[1] = sin(psip_b) * cos(theta_);
    R[0][0] = -cos(thetap);
    R[0][2] = sin(thetap);
    R[2][0] = sin(thetap);
    R[2][2] = cos(thetap);
    for (int k = 0; k < 3; k++) dr[k] = 0.0;
    for (int jj = 0; jj < 3; jj++)
      for (int k = 0; k < 3; k++) dr[k] += R[k][jj] * drp[jj];
    eph[0] = -sin(phi_o - phip);
    eph[1] = cos(phi_o - phip);
    double aaa = 0.0, rrr = 0.0;
    for (int k = 0; k < 3; k++) {
      rrr += dr[k] * dr[k];
      aaa += dr[k] * eph[k];
    }
    aaa = aaa / sqrt(rrr);
    if (aaa > 1.0) aaa = 1.0;
    if (aaa < -1.0) aaa = -1.0;
    double psitmp = acos(aaa);
    if (dr[2] < 0) psitmp = -psitmp;
    const double psi_o = (fmod(psitmp + SG_D2PI / 4.0 + 2.0 * SG_D2PI, SG_D2PI)) - SG_D2PI / 2.0;
    // detector (ra, dec) and the pixelisation (sanepic.cc:746-752, 855-874)
    const double ra_rad = phi_o;
    const double dec_rad = SG_D2PI / 4.0 - theta_o;
    const double theta = SG_D2PI / 4.0 - dec_rad;
    const double phi = fmod(ra_rad + SG_D2PI, SG_D2PI);
    int pix;
    if (theta != theta || phi != phi) {
      pix = -1;  // NaN pointing: the host applies the previous-pixel rule
    } else if (theta < 0. || theta > 3.14159265358979323846) {
      pix = -2;
      atomicExch(a.error_flag, 1);
    } else {
      pix = ang2pix_ring_dev(a.nside, theta, phi);
      if (pix < 0 || pix > 12 * (int)a.nside * (int)a.nside - 1) pix = -1;
    }
    a.ring_pix[e] = pix;
    a.psio[e] = psi_o;
  }
}

cudaError_t pointing_launch(const PointingArgs& a, cudaStream_t st) {
  const long long total = a.ns * a.nseg * (long long)a.ngroups;
  long long blocks = (total + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  k_pointing<<<(unsigned)blocks, 256, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace sg
