// FP64 pipeline: the reference's scattering path with every amplitude in
// double, the drop-in for its -DDOUBLE_PRECISION build (include/Datatypes.h:
// 33-46) and the on-GPU FP64 check of the FP32 engine.
//
// The discrete decisions are made in float, exactly as the FP32 kernels make
// them (which pixel is NaN, which Ewald plane is read, which rotated pixel is
// written: ewald_geometry, warp_tap), so the NaN masks equal the FP32 path's.
// Every amplitude is double: the dielectric tensor from the optical constants
// (include/uniaxial.h:58-169 Euler, :184-292 vector), the Hanning window
// (src/cudaMain.cu:276-295), the 3D FFT (forward, unnormalised, double
// twiddles), the DC replacement (:123-176), the intensity |(k^2 I - Q Q^T) p|^2
// (include/cudaUtils.h:268-296), the plane interpolation, the bilinear blend of
// the rotation and detector warps, and the angle sum and mean (:877-909).
//
// Schedule, per energy: LAB frame - the 5 (6 with a tilted k) distinct
// entries of Nt are transformed once and every E angle's p = Nt E / 4pi is
// formed at the Ewald sample points (exact by linearity); MATERIAL frame -
// p = R^T Nt R x per angle, 3 transforms per angle, as the reference does.
#pragma once

#include "kernels.cuh"

namespace cyr {

__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

// Refractive indices of one energy, n = 1 - delta + i beta (include/PyClass/RefractiveIndex.h:101-106).
struct Mat64 {
  double2 npar[kMaxMaterials];
  double2 nper[kMaxMaterials];
};

struct Build64Params {
  const void *vox;          // [M][V] float4 (the FP32 path's input) or double4 (vox_fp64)
  uint32_t vox_fp64;
  uint32_t nx, ny, nz, nmat;
  size_t nvox;
  uint32_t morphology;      // 0 Euler, 1 vector
  uint32_t mode;            // 0: Nt entries xx xy xz yy yz [zz]; 1: p for E (R^T p in the MATERIAL frame)
  uint32_t nvol;
  uint32_t material_frame;
  double E[3];
  double R[9];              // row major
  const double *hann_x, *hann_y, *hann_z;  // null: no window
  double2 *out;             // [nvol][V]
};

__device__ __forceinline__ void load_s64(const Build64Params &p, uint32_t m, size_t i, double s[4]) {
  if (p.vox_fp64) {
    const double4_16a v = static_cast<const double4_16a *>(p.vox)[size_t(m) * p.nvox + i];
    s[0] = v.x, s[1] = v.y, s[2] = v.z, s[3] = v.w;
  } else {
    const float4 v = static_cast<const float4 *>(p.vox)[size_t(m) * p.nvox + i];
    s[0] = v.x, s[1] = v.y, s[2] = v.z, s[3] = v.w;
  }
}

// The six entries of Nr - phi I summed over materials, in the reference's form.
__device__ void nt64(const Build64Params &p, const Mat64 &mt, size_t i, double2 nt[6]) {
  for (int q = 0; q < 6; ++q) nt[q] = make_double2(0.0, 0.0);
  for (uint32_t m = 0; m < p.nmat; ++m) {
    double s[4];
    load_s64(p, m, i, s);
    const double2 np = mt.npar[m], nq = mt.nper[m];
    const double2 npar2 = zmul(np, np), nper2 = zmul(nq, nq);
    const double2 nsum = make_double2(np.x + 2.0 * nq.x, np.y + 2.0 * nq.y);
    const double2 nsum2 = zmul(nsum, nsum);
    double sx, sy, sz, phi_a, phi_ui, phi;
    if (p.morphology == 0) {  // Euler: (S, theta, psi, Vfrac)
      double st, ct, sp, cp;
      sincos(s[1], &st, &ct);
      sincos(s[2], &sp, &cp);
      sx = cp * st, sy = sp * st, sz = ct;
      phi_a = s[3] * s[0];
      phi_ui = s[3] - phi_a;
      phi = s[3];
    } else {  // vector: (sx, sy, sz, phi_unaligned), Vfrac = |s|^2 + phi_ui
      sx = s[0], sy = s[1], sz = s[2];
      phi_ui = s[3];
      phi = phi_ui + sx * sx + sy * sy + sz * sz;
      phi_a = 1.0;
    }
    const double2 iso = zscale(nsum2, phi_ui / 9.0);
    const double2 dn = zsub(npar2, nper2);
    const double sq[3] = {sx * sx, sy * sy, sz * sz};
    const int diag[3] = {0, 3, 5};
    for (int a = 0; a < 3; ++a) {
      const double2 t = zadd(zscale(npar2, sq[a]), zscale(nper2, sq[(a + 1) % 3] + sq[(a + 2) % 3]));
      nt[diag[a]] = zadd(nt[diag[a]], make_double2(phi_a * t.x + iso.x - phi, phi_a * t.y + iso.y));
    }
    nt[1] = zadd(nt[1], zscale(dn, phi_a * sx * sy));
    nt[2] = zadd(nt[2], zscale(dn, phi_a * sx * sz));
    nt[4] = zadd(nt[4], zscale(dn, phi_a * sy * sz));
  }
}

__global__ void __launch_bounds__(256) k64_build(Build64Params p, const Mat64 *__restrict__ mat) {
  const double inv4pi = 0.25 / 3.141592653589793238462643383279502884;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < p.nvox; i += size_t(gridDim.x) * blockDim.x) {
    double2 nt[6];
    nt64(p, *mat, i, nt);
    double w = 1.0;
    if (p.hann_x) {
      const uint32_t X = uint32_t(i % p.nx), Y = uint32_t((i / p.nx) % p.ny), Z = uint32_t(i / (size_t(p.nx) * p.ny));
      w = p.hann_x[X] * p.hann_y[Y] * p.hann_z[Z];
    }
    if (p.mode == 0) {
      for (uint32_t v = 0; v < p.nvol; ++v) p.out[size_t(v) * p.nvox + i] = zscale(nt[v], inv4pi * w);
      continue;
    }
    const double *E = p.E;
    double2 q[3];
    q[0] = zadd(zadd(zscale(nt[0], E[0]), zscale(nt[1], E[1])), zscale(nt[2], E[2]));
    q[1] = zadd(zadd(zscale(nt[1], E[0]), zscale(nt[3], E[1])), zscale(nt[4], E[2]));
    q[2] = zadd(zadd(zscale(nt[2], E[0]), zscale(nt[4], E[1])), zscale(nt[5], E[2]));
    for (int c = 0; c < 3; ++c) q[c] = zscale(q[c], inv4pi);
    if (p.material_frame) {  // p <- R^T p (rotate<true>, include/Rotation.h:371-394)
      double2 r[3];
      for (int a = 0; a < 3; ++a)
        r[a] = zadd(zadd(zscale(q[0], p.R[0 * 3 + a]), zscale(q[1], p.R[1 * 3 + a])), zscale(q[2], p.R[2 * 3 + a]));
      q[0] = r[0], q[1] = r[1], q[2] = r[2];
    }
    for (int c = 0; c < 3; ++c) p.out[size_t(c) * p.nvox + i] = zscale(q[c], w);
  }
}

// ---------------------------------------------------------------------------
// FP64 FFT: shared-memory Stockham autosort, any 7-smooth length up to 4096,
// radices 8/4/2/3/5/7 with a direct DFT per radix from a double twiddle
// table W_n^m.  tx lines per block: rows along x, or tx adjacent columns for
// lines along y and z.
// ---------------------------------------------------------------------------
struct Fft64Params {
  double2 *data;
  uint32_t nx, ny, nz;
  size_t vstride;           // elements between volumes (blockIdx.y)
  uint32_t n, tx, nstages;
  uint64_t radix_code;      // radix of stage s in bits [4s, 4s+4)
  const double2 *tw;        // W_n^m
};

// One Stockham stage of radix R over tx lines of n: group j of line l reads
// x_q = src[j + q m] (m = n / R), twiddles x_q by W^(q k n / (ns R)) with
// k = j mod ns, takes its R-point DFT and writes element o to
// dst[(j / ns) ns R + k + o ns].
template <uint32_t R>
__device__ __forceinline__ void stage64(const double2 *__restrict__ src, double2 *__restrict__ dst, uint32_t n,
                                        uint32_t tx, uint32_t ns, const double2 *__restrict__ tw) {
  const uint32_t m = n / R, tstep = n / (ns * R);
  for (uint32_t g = threadIdx.x; g < tx * m; g += blockDim.x) {
    const uint32_t l = g / m, j = g % m, k = j % ns;
    const double2 *sl = src + size_t(l) * n;
    double2 x[R];
#pragma unroll
    for (uint32_t q = 0; q < R; ++q) {
      x[q] = sl[j + q * m];
      if (q && k) x[q] = zmul(x[q], tw[q * k * tstep]);
    }
    double2 *dl = dst + size_t(l) * n + (j / ns) * ns * R + k;
#pragma unroll
    for (uint32_t o = 0; o < R; ++o) {
      double2 acc = x[0];
#pragma unroll
      for (uint32_t q = 1; q < R; ++q) acc = zadd(acc, zmul(x[q], tw[((o * q) % R) * m]));
      dl[o * ns] = acc;
    }
  }
}

template <int AXIS>
__global__ void __launch_bounds__(256) k64_fft(Fft64Params p) {
  extern __shared__ double2 zsm[];
  const uint32_t n = p.n, TX = p.tx;
  double2 *bufa = zsm, *bufb = zsm + size_t(n) * TX;
  size_t base;
  uint32_t valid, lstep, estep;
  if (AXIS == 0) {
    const uint32_t rows = p.ny * p.nz, r0 = blockIdx.x * TX;
    base = size_t(r0) * p.nx;
    valid = min(TX, rows - r0);
    lstep = p.nx, estep = 1;
  } else {
    const uint32_t nxt = (p.nx + TX - 1) / TX;
    const uint32_t x0 = (blockIdx.x % nxt) * TX, other = blockIdx.x / nxt;
    valid = min(TX, p.nx - x0);
    lstep = 1;
    if (AXIS == 1) {
      base = size_t(other) * p.nx * p.ny + x0;
      estep = p.nx;
    } else {
      base = size_t(other) * p.nx + x0;
      estep = p.nx * p.ny;
    }
  }
  double2 *tile = p.data + size_t(blockIdx.y) * p.vstride + base;
  const uint32_t total = n * TX;
  for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
    uint32_t l, i;
    if (AXIS == 0) {
      l = t / n, i = t % n;
    } else {
      l = t % TX, i = t / TX;
    }
    bufa[size_t(l) * n + i] = l < valid ? tile[size_t(l) * lstep + size_t(i) * estep] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  double2 *src = bufa, *dst = bufb;
  uint32_t ns = 1;
  for (uint32_t s = 0; s < p.nstages; ++s) {
    const uint32_t R = uint32_t((p.radix_code >> (4 * s)) & 15u);
    switch (R) {
      case 2: stage64<2>(src, dst, n, TX, ns, p.tw); break;
      case 3: stage64<3>(src, dst, n, TX, ns, p.tw); break;
      case 4: stage64<4>(src, dst, n, TX, ns, p.tw); break;
      case 5: stage64<5>(src, dst, n, TX, ns, p.tw); break;
      case 7: stage64<7>(src, dst, n, TX, ns, p.tw); break;
      default: stage64<8>(src, dst, n, TX, ns, p.tw); break;
    }
    __syncthreads();
    double2 *t = src;
    src = dst, dst = t;
    ns *= R;
  }
  for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
    uint32_t l, i;
    if (AXIS == 0) {
      l = t / n, i = t % n;
    } else {
      l = t % TX, i = t / TX;
    }
    if (l < valid) tile[size_t(l) * lstep + size_t(i) * estep] = src[size_t(l) * n + i];
  }
}

// Bin 0 of each volume <- mean of its 6 (4 in 2D) periodic neighbours (src/cudaMain.cu:123-176).
__global__ void k64_dc(double2 *spec, uint32_t nvol, size_t vstride, uint32_t nx, uint32_t ny, uint32_t nz) {
  const uint32_t v = threadIdx.x;
  if (v >= nvol) return;
  double2 *V = spec + size_t(v) * vstride;
  const size_t P = size_t(nx) * ny;
  double2 s = zadd(zadd(V[1], V[nx]), zadd(V[nx - 1], V[size_t(ny - 1) * nx]));
  double cnt = 4.0;
  if (nz > 1) {
    s = zadd(s, zadd(V[P], V[size_t(nz - 1) * P]));
    cnt = 6.0;
  }
  V[0] = zscale(s, 1.0 / cnt);
}

// Ewald projection in double for every E angle: per detector pixel, the float
// geometry of ewald_geometry, the volumes gathered at the plane(s), per angle
// p_c = sum_b E_b vol[c][b], the intensity at each plane and the linear
// interpolation (1 - d) I0 + d I1 with d formed in double from the float
// plane position (include/uniaxial.h:876-947).  images[a][P] (double).
struct Ewald64Params {
  const double2 *spec;
  size_t vstride;
  uint32_t nbasis;
  uint32_t vol[3][3];
  EwaldGeom g;
  const float *qx, *qy, *qz;
  uint32_t nangles;
  const double *E;          // [nangles][nbasis] (MATERIAL frame: nbasis 1, coefficient 1)
  double *images;           // [nangles][P]
};

__global__ void __launch_bounds__(256) k64_ewald(Ewald64Params p) {
  const EwaldGeom &g = p.g;
  const size_t npix = size_t(g.nx) * g.ny;
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  const uint32_t Y = uint32_t(t / g.nx), X = uint32_t(t % g.nx);
  uint32_t zs[2];
  float w1f;
  int nplanes;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  if (!ewald_geometry(g, X, Y, zs[0], zs[1], w1f, nplanes)) {
    for (uint32_t a = 0; a < p.nangles; ++a) p.images[size_t(a) * npix + t] = nan;
    return;
  }
  // plane weight in double from the float plane position, as the reference's FP64 interpolation
  double w1 = 0.0;
  if (nplanes == 2) {
    const float posx = __fadd_rn(g.start, __fmul_rn(float(X), g.dx));
    const float posy = __fadd_rn(g.start, __fmul_rn(float(Y), g.dy));
    const float ax = __fadd_rn(g.kx, posx), ay = __fadd_rn(g.ky, posy);
    const float val = __fsub_rn(__fsub_rn(__fmul_rn(g.kmag, g.kmag), __fmul_rn(ax, ax)), __fmul_rn(ay, ay));
    const float posz = __fadd_rn(-g.kz, __fsqrt_rn(val));
    w1 = (double(posz) - (double(g.start) + double(__fmul_rn(float(zs[0]), g.dz)))) / double(g.dz);
  }
  const uint32_t ux = igor(X, g.nx), uy = igor(Y, g.ny);
  double2 P[2][3][3];
  double Q[2][3];
  for (int pl = 0; pl < nplanes; ++pl) {
    const uint32_t uz = g.twod ? 0u : igor(zs[pl], g.nz);
    const size_t idx = size_t(ux) + size_t(uy) * g.nx + size_t(uz) * g.nx * g.ny;
    for (uint32_t b = 0; b < p.nbasis; ++b)
      for (int c = 0; c < 3; ++c) P[pl][c][b] = p.spec[size_t(p.vol[c][b]) * p.vstride + idx];
    Q[pl][0] = double(g.kx) + double(p.qx[X]);
    Q[pl][1] = double(g.ky) + double(p.qy[Y]);
    Q[pl][2] = double(g.kz) + (g.twod ? 0.0 : double(p.qz[zs[pl]]));
  }
  const double d = double(g.kmag) * double(g.kmag);
  for (uint32_t a = 0; a < p.nangles; ++a) {
    const double *E = p.E + size_t(a) * p.nbasis;
    double I[2] = {0.0, 0.0};
    for (int pl = 0; pl < nplanes; ++pl) {
      double2 pc[3];
      for (int c = 0; c < 3; ++c) {
        pc[c] = make_double2(0.0, 0.0);
        for (uint32_t b = 0; b < p.nbasis; ++b) pc[c] = zadd(pc[c], zscale(P[pl][c][b], E[b]));
      }
      const double *q = Q[pl];
      const double2 qp = zadd(zadd(zscale(pc[0], q[0]), zscale(pc[1], q[1])), zscale(pc[2], q[2]));
      double r = 0.0;
      for (int c = 0; c < 3; ++c) {
        const double2 tt = zsub(zscale(pc[c], d), zscale(qp, q[c]));
        r += tt.x * tt.x + tt.y * tt.y;
      }
      I[pl] = r;
    }
    p.images[size_t(a) * npix + t] = nplanes == 2 ? (1.0 - w1) * I[0] + w1 * I[1] : I[0];
  }
}

// Bilinear blend in double at NPP's float sample position.
__device__ __forceinline__ bool warp_sample64(const double *__restrict__ src, int W, int H, const WarpCoef &c, int xd,
                                              int yd, double &out) {
  WarpTap tp;
  if (!warp_tap(W, H, c, xd, yd, tp)) return false;
  const double fx = tp.fx, fy = tp.fy;
  const double A = src[size_t(tp.y0) * W + tp.x0], B = src[size_t(tp.y0) * W + tp.x1];
  const double C = src[size_t(tp.y1) * W + tp.x0], D = src[size_t(tp.y1) * W + tp.x1];
  out = (1.0 - fy) * ((1.0 - fx) * A + fx * B) + fy * ((1.0 - fx) * C + fx * D);
  return true;
}

// Rotation of every angle's image (NaN prefill), mask, sum and mean in double
// (src/cudaMain.cu:830-909, include/uniaxial.h:958-992).
struct Rotate64Params {
  const double *images;     // [nangles][P]
  const WarpCoef *coef;     // [nangles]
  int W, H;
  uint32_t nangles, rot_mask;
  double *avg;              // [P]
};

__global__ void __launch_bounds__(256) k64_rotate_average(Rotate64Params p) {
  const size_t npix = size_t(p.W) * p.H;
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  const int xd = int(t % p.W), yd = int(t / p.W);
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  double sum = 0.0;
  uint32_t count = 0;
  for (uint32_t a = 0; a < p.nangles; ++a) {
    double v = nan;
    warp_sample64(p.images + size_t(a) * npix, p.W, p.H, p.coef[a], xd, yd, v);
    if (p.rot_mask) {
      if (isnan(v)) continue;
      ++count;
    }
    sum += v;
  }
  p.avg[t] = p.rot_mask ? (count == 0 ? 0.0 : sum / double(count)) : sum / double(p.nangles);
}

// Detector warp (src/cudaMain.cu:916-960): dst holds the prefill; written where the source falls inside.
__global__ void k64_warp(const double *__restrict__ src, double *__restrict__ dst, int W, int H, WarpCoef c,
                         double prefill) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= size_t(W) * H) return;
  double v;
  dst[t] = warp_sample64(src, W, H, c, int(t % W), int(t / W), v) ? v : prefill;
}

}  // namespace cyr
