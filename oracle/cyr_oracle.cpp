// CPU oracle for the CyRSoXS scattering path: an FP64, OpenMP restatement of the
// reference's per-energy, per-E-angle pipeline (usnistgov/cyrsoxs v1.2.0.0).
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
// legs of bench.py may load this library, and only as the checker or the timed
// CPU baseline.  The product (cyrsoxs_gb300) never calls it.
//
// Pinning: the oracle's outputs are compared against golden vectors produced by
// running the reference's own CUDA path (FP32 and FP64 builds) on a GB300
// (tests/golden/make_reference_golden.py, tests/test_oracle_golden.py).
//
// The restatement follows the reference line by line where the arithmetic is
// a discrete decision (which Ewald plane, which pixel is NaN): those are done
// in float exactly as the reference writes them, because a different rounding
// there changes the NaN mask.  Every amplitude (polarization, FFT, intensity,
// interpolation, angle sum) is computed in double.
//
// Algorithm, per energy j, per k-vector, per E-angle i (src/cudaMain.cu:586-971):
//   E-rotation matrix             include/Rotation.h:474-484
//   polarization p = Nt E / 4pi   include/uniaxial.h:58-169 (Euler), :184-292 (vector),
//                                 :305-521 (Nt, Algorithm 1), Hanning src/cudaMain.cu:276-295
//   forward unnormalised 3D DFT   include/cudaMain.h:184-190 (cufftExecC2C, FORWARD)
//   DC <- mean of 6 (4) neighbours src/cudaMain.cu:123-176
//   "Igor" shift j -> N/2 - j     include/uniaxial.h:570-613
//   Ewald projection              include/uniaxial.h:876-947 (PARTIAL), :821-874 (FULL),
//                                 intensity include/cudaUtils.h:268-296
//   rotate by the E angle         src/cudaMain.cu:830-875 (NPP bilinear warp, NaN prefill)
//   mask / sum / average          src/cudaMain.cu:877-909, include/uniaxial.h:958-992
//   detector warp                 src/cudaMain.cu:916-960, include/Rotation.h:499-516
//   output [E][K][Ny][Nx]         src/cudaMain.cu:968-971

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using cd = std::complex<double>;
constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------------------
// Rotation math in float, as the reference computes it (include/Rotation.h).
// ---------------------------------------------------------------------------
struct F3 {
  float x, y, z;
};
struct FM {
  float m[9];
  FM() { std::memset(m, 0, sizeof m); }
  float &at(int i, int j) { return m[3 * i + j]; }
  float at(int i, int j) const { return m[3 * i + j]; }
};

inline bool fequals(float a, float b) { return std::fabs(a - b) < 1e-6; }  // FEQUALS, Datatypes.h:151
inline float dotf(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline F3 crossf(F3 a, F3 b) {  // Rotation.h:187-193
  return {a.y * b.z - a.z * b.y, -(a.x * b.z - a.z * b.x), a.x * b.y - a.y * b.x};
}
inline float normf(F3 v) { return std::sqrt(dotf(v, v)); }
inline FM identity() {
  FM r;
  r.at(0, 0) = r.at(1, 1) = r.at(2, 2) = 1.f;
  return r;
}
inline FM matmul(const FM &a, const FM &b) {  // Matrix::performMatrixMultiplication<false,false>
  FM r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) r.m[i * 3 + j] += a.m[i * 3 + k] * b.m[k * 3 + j];
  return r;
}
inline F3 matvec(const FM &a, F3 v) {  // doMatVec<false>, Rotation.h:348-360
  return {a.at(0, 0) * v.x + a.at(0, 1) * v.y + a.at(0, 2) * v.z, a.at(1, 0) * v.x + a.at(1, 1) * v.y + a.at(1, 2) * v.z,
          a.at(2, 0) * v.x + a.at(2, 1) * v.y + a.at(2, 2) * v.z};
}
FM inverse(const FM &a) {  // computeInverseMatrix, Rotation.h:228-247 (det in double, 1/det in float)
  const double det = a.at(0, 0) * (a.at(1, 1) * a.at(2, 2) - a.at(2, 1) * a.at(1, 2)) -
                     a.at(0, 1) * (a.at(1, 0) * a.at(2, 2) - a.at(1, 2) * a.at(2, 0)) +
                     a.at(0, 2) * (a.at(1, 0) * a.at(2, 1) - a.at(1, 1) * a.at(2, 0));
  const float inv = static_cast<float>(1. / det);
  FM r;
  r.at(0, 0) = (a.at(1, 1) * a.at(2, 2) - a.at(2, 1) * a.at(1, 2)) * inv;
  r.at(0, 1) = (a.at(0, 2) * a.at(2, 1) - a.at(0, 1) * a.at(2, 2)) * inv;
  r.at(0, 2) = (a.at(0, 1) * a.at(1, 2) - a.at(0, 2) * a.at(1, 1)) * inv;
  r.at(1, 0) = (a.at(1, 2) * a.at(2, 0) - a.at(1, 0) * a.at(2, 2)) * inv;
  r.at(1, 1) = (a.at(0, 0) * a.at(2, 2) - a.at(0, 2) * a.at(2, 0)) * inv;
  r.at(1, 2) = (a.at(1, 0) * a.at(0, 2) - a.at(0, 0) * a.at(1, 2)) * inv;
  r.at(2, 0) = (a.at(1, 0) * a.at(2, 1) - a.at(2, 0) * a.at(1, 1)) * inv;
  r.at(2, 1) = (a.at(2, 0) * a.at(0, 1) - a.at(0, 0) * a.at(2, 1)) * inv;
  r.at(2, 2) = (a.at(0, 0) * a.at(1, 1) - a.at(1, 0) * a.at(0, 1)) * inv;
  return r;
}
// Matrix taking a onto b: F G F^-1 (Rotation.h:272-315).
FM align(F3 a, F3 b) {
  if (fequals(a.x, b.x) && fequals(a.y, b.y) && fequals(a.z, b.z)) return identity();
  const float d = dotf(a, b);
  const F3 c = crossf(a, b);
  const float nc = normf(c);
  FM G;
  G.at(0, 0) = d;
  G.at(0, 1) = -nc;
  G.at(1, 0) = nc;
  G.at(1, 1) = d;
  G.at(2, 2) = 1.f;
  const F3 sub{b.x - d * a.x, b.y - d * a.y, b.z - d * a.z};
  const float ns = normf(sub);
  FM F;
  F.at(0, 0) = a.x;
  F.at(1, 0) = a.y;
  F.at(2, 0) = a.z;
  F.at(0, 1) = sub.x / ns;
  F.at(1, 1) = sub.y / ns;
  F.at(2, 1) = sub.z / ns;
  F.at(0, 2) = -c.x;
  F.at(1, 2) = -c.y;
  F.at(2, 2) = -c.z;
  return matmul(F, matmul(G, inverse(F)));
}
F3 rodrigues(F3 v, F3 axis, float angle) {  // Rotation.h:326-338
  const float ca = std::cos(angle), sa = std::sin(angle);
  const F3 cr = crossf(axis, v);
  const float dp = dotf(axis, v);
  const float s3 = (1 - ca) * dp;
  return {ca * v.x + sa * cr.x + s3 * axis.x, ca * v.y + sa * cr.y + s3 * axis.y, ca * v.z + sa * cr.z + s3 * axis.z};
}
// computeRotationMatrixBaseConfiguration (Rotation.h:422-465): the angle about k
// that brings R_k x onto the x-z plane with positive x.
float base_angle(F3 k, const FM &rk) {
  constexpr uint32_t n = 100000;
  constexpr float dtheta = static_cast<float>(kPi / (n * 1.0));
  const F3 sx = matvec(rk, {1.f, 0.f, 0.f});
  float best = std::numeric_limits<float>::infinity(), ang = 0.f;
  for (uint32_t i = 0; i < n; ++i) {
    const F3 r = rodrigues(sx, k, i * dtheta);
    const float diff = std::fabs(r.y);
    if (best > diff) {
      best = diff;
      ang = i * dtheta;
    }
  }
  const F3 r = rodrigues(sx, k, ang);
  return r.x > 0 ? ang : static_cast<float>(ang + kPi);
}
// computeRotationMatrix(k, R_k, R, angle), Rotation.h:474-484.
FM e_rotation(F3 k, const FM &rk, float angle) {
  const F3 sx = matvec(rk, {1.f, 0.f, 0.f});
  const F3 rx = rodrigues(sx, k, angle);
  return matmul(align(sx, rx), rk);
}
F3 normalized(F3 v) {  // normalizeVec, Rotation.h:490-493
  const float n = normf(v);
  const float s = static_cast<float>(1. / n);
  return {s * v.x, s * v.y, s * v.z};
}
// computeWarpAffineMatrix, Rotation.h:499-516 (double).
void warp_affine_from_points(const double s[3][2], const double d[3][2], double c[2][3]) {
  const double x0 = s[0][0], y0 = s[0][1], x1 = s[1][0], y1 = s[1][1], x2 = s[2][0], y2 = s[2][1];
  const double u0 = d[0][0], v0 = d[0][1], u1 = d[1][0], v1 = d[1][1], u2 = d[2][0], v2 = d[2][1];
  const double den = x0 * y1 - x1 * y0 - x0 * y2 + x2 * y0 + x1 * y2 - x2 * y1;
  c[0][0] = (u0 * y1 - u1 * y0 - u0 * y2 + u2 * y0 + u1 * y2 - u2 * y1) / den;
  c[0][1] = -(u0 * x1 - u1 * x0 - u0 * x2 + u2 * x0 + u1 * x2 - u2 * x1) / den;
  c[0][2] = (u0 * x1 * y2 - u0 * x2 * y1 - u1 * x0 * y2 + u1 * x2 * y0 + u2 * x0 * y1 - u2 * x1 * y0) / den;
  c[1][0] = (v0 * y1 - v1 * y0 - v0 * y2 + v2 * y0 + v1 * y2 - v2 * y1) / den;
  c[1][1] = -(v0 * x1 - v1 * x0 - v0 * x2 + v2 * x0 + v1 * x2 - v2 * x1) / den;
  c[1][2] = (v0 * x1 * y2 - v0 * x2 * y1 - v1 * x0 * y2 + v1 * x2 * y0 + v2 * x0 * y1 - v2 * x1 * y0) / den;
}

// ---------------------------------------------------------------------------
// FP64 FFT: recursive mixed-radix decimation in time, exact DFT for each prime
// factor, double twiddles.  Forward, unnormalised (the cuFFT convention the
// reference uses, include/cudaMain.h:184-190).
// ---------------------------------------------------------------------------
struct Plan {
  int n = 0;
  std::vector<int> radix;
  std::vector<cd> w;  // w[m] = exp(-2 pi i m / n)
  explicit Plan(int n_) : n(n_), w(n_) {
    int r = n;
    for (int p : {4, 2, 3, 5, 7}) {
      while (r % p == 0 && (p != 4 || r % 4 == 0)) {
        radix.push_back(p);
        r /= p;
      }
    }
    for (int p = 11; r > 1; p += 2)
      while (r % p == 0) {
        radix.push_back(p);
        r /= p;
      }
    for (int m = 0; m < n; ++m) w[m] = std::polar(1.0, -2.0 * kPi * m / n);
  }
};

void fft_rec(const cd *in, cd *out, int len, int stride, const Plan &p, size_t lvl, std::vector<cd> &tmp) {
  if (len == 1) {
    out[0] = in[0];
    return;
  }
  const int r = p.radix[lvl], m = len / r, scale = p.n / len;
  for (int j = 0; j < r; ++j) fft_rec(in + j * stride, out + j * m, m, stride * r, p, lvl + 1, tmp);
  cd t[64];
  std::vector<cd> big;
  cd *tt = t;
  if (r > 64) {
    big.resize(r);
    tt = big.data();
  }
  for (int k = 0; k < m; ++k) {
    for (int j = 0; j < r; ++j) tt[j] = out[j * m + k] * p.w[(size_t(j) * k * scale) % p.n];
    for (int q = 0; q < r; ++q) {
      cd s = 0;
      for (int j = 0; j < r; ++j) s += tt[j] * p.w[(size_t(j) * q * m * scale) % p.n];
      tmp[q] = s;
    }
    for (int q = 0; q < r; ++q) out[q * m + k] = tmp[q];
  }
}

void fft1d(const Plan &p, cd *line, std::vector<cd> &work, std::vector<cd> &tmp) {
  std::copy(line, line + p.n, work.begin());
  fft_rec(work.data(), line, p.n, 1, p, 0, tmp);
}

// In-place 3D forward DFT of a [nz][ny][nx] volume.
void fft3d(cd *v, int nx, int ny, int nz) {
  const int dims[3] = {nx, ny, nz};
  const size_t strides[3] = {1, size_t(nx), size_t(nx) * ny};
  for (int ax = 0; ax < 3; ++ax) {
    const int n = dims[ax];
    if (n == 1) continue;
    const Plan p(n);
    const size_t s = strides[ax];
    const size_t nlines = size_t(nx) * ny * nz / n;
#pragma omp parallel
    {
      std::vector<cd> line(n), work(n), tmp(std::max(64, n));
#pragma omp for schedule(static)
      for (long long li = 0; li < static_cast<long long>(nlines); ++li) {
        // line li: enumerate the (other two) coordinates
        size_t base;
        if (ax == 0) {
          base = size_t(li) * nx;
        } else if (ax == 1) {
          const size_t x = size_t(li) % nx, z = size_t(li) / nx;
          base = z * size_t(nx) * ny + x;
        } else {
          base = size_t(li);
        }
        for (int i = 0; i < n; ++i) line[i] = v[base + i * s];
        fft1d(p, line.data(), work, tmp);
        for (int i = 0; i < n; ++i) v[base + i * s] = line[i];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Case description (the layout tests/golden/cases.py writes).
// ---------------------------------------------------------------------------
struct Case {
  uint32_t nx, ny, nz, nmat, ne, nk;
  uint32_t morph, window, interp, scatter, rotmask, algo, streams, frame, casetype, mode;
  float phys, a0, a1, da, pol_energy, pol_eangle;
  float det[3];
  std::vector<float> energies, kvecs, optical, vox;
  const float *voxp = nullptr;  // the voxel array in use (vox.data() or caller memory)
};

Case read_case(const char *path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw std::runtime_error(std::string("cannot open ") + path);
  char magic[8];
  in.read(magic, 8);
  if (std::memcmp(magic, "CYRCASE1", 8) != 0) throw std::runtime_error("bad case magic");
  Case c;
  uint32_t u[16];
  in.read(reinterpret_cast<char *>(u), sizeof u);
  c.nx = u[0], c.ny = u[1], c.nz = u[2], c.nmat = u[3], c.ne = u[4], c.nk = u[5];
  c.morph = u[6], c.window = u[7], c.interp = u[8], c.scatter = u[9], c.rotmask = u[10], c.algo = u[11];
  c.streams = u[12], c.frame = u[13], c.casetype = u[14], c.mode = u[15];
  float f[9];
  in.read(reinterpret_cast<char *>(f), sizeof f);
  c.phys = f[0], c.a0 = f[1], c.a1 = f[2], c.da = f[3], c.pol_energy = f[4], c.pol_eangle = f[5];
  c.det[0] = f[6], c.det[1] = f[7], c.det[2] = f[8];
  auto rd = [&](std::vector<float> &v, size_t n) {
    v.resize(n);
    in.read(reinterpret_cast<char *>(v.data()), n * 4);
  };
  rd(c.energies, c.ne);
  rd(c.kvecs, size_t(c.nk) * 3);
  rd(c.optical, size_t(c.ne) * c.nmat * 4);
  rd(c.vox, size_t(c.nmat) * c.nx * c.ny * c.nz * 4);
  if (!in) throw std::runtime_error("truncated case file");
  c.voxp = c.vox.data();
  return c;
}

// The E-angle schedule: InputData::setEAngles (InputData.h:493-512) and
// src/cudaMain.cu:393-394.
void angle_schedule(const Case &c, float &start, float &inc, uint32_t &n) {
  start = c.a0;
  inc = c.da;
  if (fequals(c.a0, c.a1)) inc = 1.0f;
  n = static_cast<uint32_t>(std::round((c.a1 - c.a0) / inc + 1));
}

// Optical constants n = 1 - delta + i beta (RefractiveIndex.h:101-106).  The
// FP32 reference forms n in float, which rounds the contrast n^2 - 1 (a few
// 1e-3) to ~5 significant digits; the oracle forms it in double, as the
// reference's FP64 build does.
struct Mat {
  cd npar, nper;
};
Mat material(const Case &c, size_t e, size_t m) {
  const float *o = &c.optical[(e * c.nmat + m) * 4];
  return {cd(1.0 - double(o[0]), o[1]), cd(1.0 - double(o[2]), o[3])};
}

// Per-voxel dielectric tensor minus phi*I, 6 entries [xx, xy, xz, yy, yz, zz],
// summed over materials (uniaxial.h:58-169 Euler, :184-292 vector).
void nt_voxel(const Case &c, const std::vector<Mat> &mats, size_t i, size_t nvox, cd nt[6]) {
  for (int q = 0; q < 6; ++q) nt[q] = 0;
  for (uint32_t m = 0; m < c.nmat; ++m) {
    const float *s = &c.voxp[(m * nvox + i) * 4];
    const cd npar2 = mats[m].npar * mats[m].npar, nper2 = mats[m].nper * mats[m].nper;
    const cd nsum = mats[m].npar + 2.0 * mats[m].nper;
    const cd nsum2 = nsum * nsum;
    double sx, sy, sz, phi_a, phi_ui, phi;
    if (c.morph == 0) {  // Euler: s1 = (S, theta, psi, Vfrac)
      const double S = s[0], th = s[1], ps = s[2], vf = s[3];
      sx = std::cos(ps) * std::sin(th);
      sy = std::sin(ps) * std::sin(th);
      sz = std::cos(th);
      phi_a = vf * S;
      phi_ui = vf - phi_a;
      phi = vf;
    } else {  // vector: s1 = (sx, sy, sz, phi_unaligned), Vfrac = |s|^2 + phi_ui
      sx = s[0], sy = s[1], sz = s[2];
      phi_ui = s[3];
      phi = phi_ui + sx * sx + sy * sy + sz * sz;
      phi_a = 1.0;
    }
    const cd iso = phi_ui * nsum2 / 9.0;
    const cd dn = npar2 - nper2;
    nt[0] += phi_a * (npar2 * sx * sx + nper2 * (sy * sy + sz * sz)) + iso - phi;
    nt[1] += phi_a * dn * sx * sy;
    nt[2] += phi_a * dn * sx * sz;
    nt[3] += phi_a * (npar2 * sy * sy + nper2 * (sx * sx + sz * sz)) + iso - phi;
    nt[4] += phi_a * dn * sy * sz;
    nt[5] += phi_a * (npar2 * sz * sz + nper2 * (sx * sx + sy * sy)) + iso - phi;
  }
}

// Polarization for one E rotation matrix (uniaxial.h:58-169 with the Hanning
// window of src/cudaMain.cu:276-295 for Algorithm 0).
void polarization(const Case &c, const std::vector<Mat> &mats, const FM &R, bool hanning, cd *px, cd *py, cd *pz) {
  const size_t nvox = size_t(c.nx) * c.ny * c.nz;
  const double E[3] = {R.at(0, 0), R.at(1, 0), R.at(2, 0)};
  const double inv4pi = 1.0 / (4.0 * kPi);
  const bool twod = c.nz == 1;
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < static_cast<long long>(nvox); ++ii) {
    const size_t i = size_t(ii);
    cd nt[6];
    nt_voxel(c, mats, i, nvox, nt);
    cd p[3] = {(nt[0] * E[0] + nt[1] * E[1] + nt[2] * E[2]) * inv4pi,
               (nt[1] * E[0] + nt[3] * E[1] + nt[4] * E[2]) * inv4pi,
               (nt[2] * E[0] + nt[4] * E[1] + nt[5] * E[2]) * inv4pi};
    if (c.frame == 0) {  // MATERIAL: p <- R^T p (rotate<true>, Rotation.h:371-394)
      cd q[3];
      for (int a = 0; a < 3; ++a) q[a] = double(R.at(0, a)) * p[0] + double(R.at(1, a)) * p[1] + double(R.at(2, a)) * p[2];
      p[0] = q[0], p[1] = q[1], p[2] = q[2];
    }
    if (hanning) {
      const size_t X = i % c.nx, Y = (i / c.nx) % c.ny, Z = i / (size_t(c.nx) * c.ny);
      double w = 0.5 * (1 - std::cos(2 * kPi * X / c.nx)) * 0.5 * (1 - std::cos(2 * kPi * Y / c.ny));
      if (!twod) w *= 0.5 * (1 - std::cos(2 * kPi * Z / c.nz));
      p[0] *= w, p[1] *= w, p[2] *= w;
    }
    px[i] = p[0], py[i] = p[1], pz[i] = p[2];
  }
}

// P[0] <- mean of its periodic neighbours (src/cudaMain.cu:123-176).
void replace_dc(cd *P, uint32_t nx, uint32_t ny, uint32_t nz) {
  cd s = P[1] + P[nx] + P[nx - 1] + P[size_t(ny - 1) * nx];
  int n = 4;
  if (nz > 1) {
    s += P[size_t(nx) * ny] + P[size_t(nz - 1) * nx * ny];
    n += 2;
  }
  P[0] = s / double(n);
}

// Shifted index -> unshifted index, per axis j -> (N/2 - j) mod N (uniaxial.h:589-605).
inline uint32_t igor(uint32_t j, uint32_t n) { return j <= n / 2 ? n / 2 - j : n + (n / 2 - j); }

// |(k^2 I - Q Q^T) p|^2 (cudaUtils.h:268-296), Q = k khat + q.
inline double intensity(const double Q[3], const cd p[3], double k) {
  const double d = k * k;
  double r = 0;
  for (int a = 0; a < 3; ++a) {
    cd t = d * p[a];
    for (int b = 0; b < 3; ++b) t -= Q[a] * Q[b] * p[b];
    r += std::norm(t);
  }
  return r;
}

// Float geometry of the Ewald projection (uniaxial.h:891-917); shared by PARTIAL and FULL.
struct EwaldGeom {
  float start, dx, dy, dz;
};
EwaldGeom ewald_geom(const Case &c) {
  EwaldGeom g;
  g.start = -static_cast<float>(kPi / c.phys);
  g.dx = static_cast<float>((2.0 * kPi / c.phys) / ((c.nx - 1) * 1.0));
  g.dy = static_cast<float>((2.0 * kPi / c.phys) / ((c.ny - 1) * 1.0));
  g.dz = c.nz == 1 ? 0.f : static_cast<float>((2.0 * kPi / c.phys) / ((c.nz - 1) * 1.0));
  return g;
}

// The q-grid point of voxel (X,Y,Z) as computeScatter3D forms it (uniaxial.h:645-650).
inline void qgrid(const Case &c, const EwaldGeom &g, uint32_t X, uint32_t Y, uint32_t Z, double q[3]) {
  q[0] = static_cast<float>((-kPi / c.phys) + X * g.dx);
  q[1] = static_cast<float>((-kPi / c.phys) + Y * g.dy);
  q[2] = c.nz == 1 ? 0.0 : static_cast<float>((-kPi / c.phys) + Z * g.dz);
}

// Ewald projection of the (unshifted) spectra onto [Ny][Nx] (uniaxial.h:876-947);
// the Igor shift is applied as index arithmetic.
void ewald(const Case &c, const EwaldGeom &g, const cd *P[3], float kmag, F3 kvec, double *proj) {
  const uint32_t nx = c.nx, ny = c.ny, nz = c.nz;
  const bool twod = nz == 1;
  const float kx = kmag * kvec.x, ky = kmag * kvec.y, kz = kmag * kvec.z;
  auto sample = [&](uint32_t X, uint32_t Y, uint32_t Z) {
    const size_t id = size_t(igor(X, nx)) + size_t(igor(Y, ny)) * nx + size_t(igor(Z, nz)) * nx * ny;
    const cd p[3] = {P[0][id], P[1][id], P[2][id]};
    double q[3];
    qgrid(c, g, X, Y, Z, q);
    const double Q[3] = {double(kx) + q[0], double(ky) + q[1], double(kz) + q[2]};
    return intensity(Q, p, kmag);
  };
#pragma omp parallel for schedule(static)
  for (long long t = 0; t < static_cast<long long>(nx) * ny; ++t) {
    const uint32_t Y = uint32_t(t / nx), X = uint32_t(t % nx);
    const float posy = g.start + Y * g.dy, posx = g.start + X * g.dx;
    const float val = kmag * kmag - (kx + posx) * (kx + posx) - (ky + posy) * (ky + posy);
    double out;
    if (val < 0 || X == nx - 1 || Y == ny - 1) {
      out = std::numeric_limits<double>::quiet_NaN();
    } else {
      const float posz = -kz + std::sqrt(val);
      if (c.interp == 0) {  // nearest neighbour: computeEquivalentID (uniaxial.h:739-753)
        uint32_t Z = 0;
        if (!twod) {
          const float r = std::round((posz - g.start) / g.dz);
          Z = r <= 0 ? 0u : static_cast<uint32_t>(r);
        }
        out = Z > nz - 1 ? std::numeric_limits<double>::quiet_NaN() : sample(X, Y, Z);
      } else if (twod) {
        out = sample(X, Y, 0);
      } else {
        const float t0 = (posz - g.start) / g.dz;
        const uint32_t Z = t0 <= 0 ? 0u : static_cast<uint32_t>(t0);  // float -> UINT saturates on the GPU
        if (Z >= nz - 1) {
          // Z > Nz-1 is the reference's NaN rule; Z == Nz-1 would make it read
          // plane Nz, outside the volume: the oracle reports NaN there.
          out = std::numeric_limits<double>::quiet_NaN();
        } else {
          const double d1 = sample(X, Y, Z), d2 = sample(X, Y, Z + 1);
          const double diff = (double(posz) - (double(g.start) + double(Z * g.dz))) / double(g.dz);
          out = (1 - diff) * d1 + diff * d2;
        }
      }
    }
    proj[t] = out;
  }
}

// Bilinear affine warp with the semantics of nppiWarpAffine_32f_C1R with
// NPPI_INTER_LINEAR, as pinned bit-for-bit by tests/golden/npp_warp_out.bin
// (49 probes: identities, sub-pixel shifts, general affines, rotations with
// NaN borders).  Destination pixel (x', y') samples the source at C^-1 (x', y'):
//   a00..a11 = float(inverse of the 2x2 part, in double)
//   a02, a12 = float(-(a00 c02 + a01 c12)) in double from the rounded a's
//   xs = fma(a00, x', a01 * y') + a02 in float (likewise ys)
// and the pixel is written only when 0 <= xs <= W-1 and 0 <= ys <= H-1;
// otherwise it keeps its prefill.  Neighbours x0+1, y0+1 are clamped to the
// image, so a zero weight on a NaN neighbour still yields NaN.  The sample
// positions (hence the NaN mask) are NPP's exactly; the interpolation itself
// is done in double here.
void npp_inverse(const double c[2][3], float a[6]) {
  const double det = c[0][0] * c[1][1] - c[0][1] * c[1][0];
  a[0] = static_cast<float>(c[1][1] / det);
  a[1] = static_cast<float>(-c[0][1] / det);
  a[3] = static_cast<float>(-c[1][0] / det);
  a[4] = static_cast<float>(c[0][0] / det);
  a[2] = static_cast<float>(-(double(a[0]) * c[0][2] + double(a[1]) * c[1][2]));
  a[5] = static_cast<float>(-(double(a[3]) * c[0][2] + double(a[4]) * c[1][2]));
}
inline float npp_coord(float a, float b, float off, float x, float y) {
  const float by = b * y;  // rounded product, then one fused multiply-add, then the offset
  return std::fma(a, x, by) + off;
}
void warp(const double *src, double *dst, int W, int H, const double c[2][3]) {
  float a[6];
  npp_inverse(c, a);
#pragma omp parallel for schedule(static)
  for (long long t = 0; t < static_cast<long long>(W) * H; ++t) {
    const int yd = int(t / W), xd = int(t % W);
    const float xs = npp_coord(a[0], a[1], a[2], float(xd), float(yd));
    const float ys = npp_coord(a[3], a[4], a[5], float(xd), float(yd));
    if (!(xs >= 0.f && xs <= float(W - 1) && ys >= 0.f && ys <= float(H - 1))) continue;
    const int x0 = std::min(int(std::floor(xs)), W - 1), y0 = std::min(int(std::floor(ys)), H - 1);
    const int x1 = std::min(x0 + 1, W - 1), y1 = std::min(y0 + 1, H - 1);
    const double fx = double(xs - float(x0)), fy = double(ys - float(y0));
    const double p = src[size_t(y0) * W + x0], b = src[size_t(y0) * W + x1];
    const double q = src[size_t(y1) * W + x0], d = src[size_t(y1) * W + x1];
    dst[t] = (1 - fy) * ((1 - fx) * p + fx * b) + fy * ((1 - fx) * q + fx * d);
  }
}

// The per-angle rotation coefficients (src/cudaMain.cu:848-855).
void rotation_coeffs(float eangle, uint32_t nx, uint32_t ny, double c[2][3]) {
  const double al = std::cos(eangle), be = std::sin(eangle);
  c[0][0] = al, c[0][1] = be, c[0][2] = static_cast<float>((1 - al) * nx / 2 - be * ny / 2.);
  c[1][0] = -be, c[1][1] = al, c[1][2] = static_cast<float>(be * nx / 2. + (1 - al) * ny / 2.);
}

std::vector<F3> kvectors(const Case &c) {
  std::vector<F3> ks;
  if (c.casetype == 0) {
    ks.push_back({0.f, 0.f, 1.f});
  } else {
    for (uint32_t i = 0; i < c.nk; ++i) ks.push_back(normalized({c.kvecs[3 * i], c.kvecs[3 * i + 1], c.kvecs[3 * i + 2]}));
  }
  return ks;
}

// Full pipeline: out[E][K][Ny][Nx].  angle_limit > 0 truncates the angle loop
// (used only to time a bounded CPU sample).
void simulate(const Case &c, double *out, uint32_t angle_limit, uint32_t energy_limit) {
  const size_t nvox = size_t(c.nx) * c.ny * c.nz, npix = size_t(c.nx) * c.ny;
  const std::vector<F3> ks = kvectors(c);
  // RotationMatrix::initComputation (src/RotationMatrix.cpp:30-51)
  std::vector<FM> rk(ks.size());
  std::vector<float> base(ks.size());
  for (size_t i = 0; i < ks.size(); ++i) {
    rk[i] = align({0.f, 0.f, 1.f}, ks[i]);
    base[i] = base_angle(ks[i], rk[i]);
  }
  const F3 det = c.casetype == 2 ? F3{c.det[0], c.det[1], c.det[2]} : F3{0.f, 0.f, 1.f};
  const FM detm = align({0.f, 0.f, 1.f}, det);
  float start, inc;
  uint32_t nang;
  angle_schedule(c, start, inc, nang);
  const uint32_t nang_run = angle_limit ? std::min(angle_limit, nang) : nang;
  const uint32_t ne_run = energy_limit ? std::min(energy_limit, c.ne) : c.ne;
  const EwaldGeom g = ewald_geom(c);
  const bool hanning = c.algo == 0 && c.window == 1;
  std::vector<cd> px(nvox), py(nvox), pz(nvox);
  std::vector<double> proj(npix), rot(npix), avg(npix), fin(npix);
  std::vector<uint32_t> mask(npix);
  const int W = int(c.ny), H = int(c.nx);  // NPP image: width = Ny, height = Nx (src/cudaMain.cu:488-496)
  for (uint32_t e = 0; e < ne_run; ++e) {
    std::vector<Mat> mats(c.nmat);
    for (uint32_t m = 0; m < c.nmat; ++m) mats[m] = material(c, e, m);
    const float energy = c.energies[e];
    const float wavelength = static_cast<float>(1239.84197 / energy);
    const float kmag = static_cast<float>(2 * kPi / wavelength);
    for (size_t ki = 0; ki < ks.size(); ++ki) {
      std::fill(avg.begin(), avg.end(), 0.0);
      std::fill(mask.begin(), mask.end(), 0u);
      for (uint32_t i = 0; i < nang_run; ++i) {
        const float eangle = static_cast<float>((base[ki] + start + i * inc) * kPi / 180.0);
        const FM R = e_rotation(ks[ki], rk[ki], eangle);
        polarization(c, mats, R, hanning, px.data(), py.data(), pz.data());
        fft3d(px.data(), c.nx, c.ny, c.nz);
        fft3d(py.data(), c.nx, c.ny, c.nz);
        fft3d(pz.data(), c.nx, c.ny, c.nz);
        replace_dc(px.data(), c.nx, c.ny, c.nz);
        replace_dc(py.data(), c.nx, c.ny, c.nz);
        replace_dc(pz.data(), c.nx, c.ny, c.nz);
        const cd *P[3] = {px.data(), py.data(), pz.data()};
        ewald(c, g, P, kmag, ks[ki], proj.data());
        double coef[2][3];
        rotation_coeffs(eangle, c.nx, c.ny, coef);
        std::fill(rot.begin(), rot.end(), std::numeric_limits<double>::quiet_NaN());
        warp(proj.data(), rot.data(), W, H, coef);
        for (size_t t = 0; t < npix; ++t) {
          double v = rot[t];
          if (c.rotmask) {
            if (std::isnan(v)) {
              v = 0;
            } else {
              mask[t]++;
            }
          }
          avg[t] += v;
        }
      }
      for (size_t t = 0; t < npix; ++t) {
        if (c.rotmask) {
          avg[t] = mask[t] == 0 ? 0.0 : avg[t] / mask[t];
        } else {
          avg[t] = avg[t] / nang_run;
        }
      }
      // detector warp (src/cudaMain.cu:916-960)
      const double sp[3][2] = {{c.nx / 2., c.ny / 2.}, {c.nx * 0.5, c.ny * 1.0}, {c.nx * 1.0, c.ny * 0.5}};
      const double ctr[2] = {c.nx / 2., c.ny / 2.};
      const FM rm = matmul(detm, rk[ki]);
      double dp[3][2];
      for (int q = 0; q < 3; ++q) {
        const F3 s{static_cast<float>(sp[q][0] - ctr[0]), static_cast<float>(sp[q][1] - ctr[1]), 0.f};
        F3 d = matvec(rm, s);
        d.x = static_cast<float>(d.x + ctr[0]);
        d.y = static_cast<float>(d.y + ctr[1]);
        dp[q][0] = d.x, dp[q][1] = d.y;
      }
      double coef[2][3];
      warp_affine_from_points(sp, dp, coef);
      std::fill(fin.begin(), fin.end(), c.rotmask ? 0.0 : std::numeric_limits<double>::quiet_NaN());
      warp(avg.data(), fin.data(), W, H, coef);
      std::copy(fin.begin(), fin.end(), out + (size_t(e) * ks.size() + ki) * npix);
    }
  }
}

thread_local std::string g_err;

}  // namespace

extern "C" {

const char *oracle_last_error() { return g_err.c_str(); }

int oracle_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// Runs a case file through the full pipeline; out holds [E][K][Ny][Nx] doubles.
// angle_limit / energy_limit > 0 truncate the loops (bounded CPU samples).
// Returns 0 on success; *seconds receives the wall time of the computation.
int oracle_run_case(const char *path, double *out, uint32_t angle_limit, uint32_t energy_limit, double *seconds) {
  try {
    const Case c = read_case(path);
    const auto t0 = std::chrono::steady_clock::now();
    simulate(c, out, angle_limit, energy_limit);
    if (seconds) seconds[0] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

// Same pipeline from arrays: hdr = {nx, ny, nz, nmat, ne, nk, morph, window,
// interp, scatter, rotmask, algo, streams, frame, casetype, mode} (u32[16]),
// fl = {phys, a0, a1, da, pol_energy, pol_eangle, det0, det1, det2} (f32[9]).
int oracle_run_arrays(const uint32_t *hdr, const float *fl, const float *energies, const float *kvecs,
                      const float *optical, const float *voxels, double *out, uint32_t angle_limit,
                      uint32_t energy_limit, double *seconds) {
  try {
    Case c;
    c.nx = hdr[0], c.ny = hdr[1], c.nz = hdr[2], c.nmat = hdr[3], c.ne = hdr[4], c.nk = hdr[5];
    c.morph = hdr[6], c.window = hdr[7], c.interp = hdr[8], c.scatter = hdr[9], c.rotmask = hdr[10];
    c.algo = hdr[11], c.streams = hdr[12], c.frame = hdr[13], c.casetype = hdr[14], c.mode = hdr[15];
    c.phys = fl[0], c.a0 = fl[1], c.a1 = fl[2], c.da = fl[3], c.pol_energy = fl[4], c.pol_eangle = fl[5];
    c.det[0] = fl[6], c.det[1] = fl[7], c.det[2] = fl[8];
    c.energies.assign(energies, energies + c.ne);
    c.kvecs.assign(kvecs, kvecs + size_t(c.nk) * 3);
    c.optical.assign(optical, optical + size_t(c.ne) * c.nmat * 4);
    c.voxp = voxels;
    const auto t0 = std::chrono::steady_clock::now();
    simulate(c, out, angle_limit, energy_limit);
    if (seconds) seconds[0] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

// The computePolarization debug path (src/cudaMain.cu:1669-1738): one energy,
// E angle in radians, kID 0; out holds px, py, pz as complex doubles [3][V].
int oracle_polarization_case(const char *path, double *out) {
  try {
    const Case c = read_case(path);
    const auto &es = c.energies;
    const size_t eid = std::lower_bound(es.begin(), es.end(), c.pol_energy) - es.begin();
    std::vector<Mat> mats(c.nmat);
    for (uint32_t m = 0; m < c.nmat; ++m) mats[m] = material(c, eid, m);
    const std::vector<F3> ks = kvectors(c);
    const FM rk = align({0.f, 0.f, 1.f}, ks[0]);
    const FM R = e_rotation(ks[0], rk, c.pol_eangle);
    const size_t nvox = size_t(c.nx) * c.ny * c.nz;
    cd *o = reinterpret_cast<cd *>(out);
    polarization(c, mats, R, c.window == 1, o, o + nvox, o + 2 * nvox);
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

// Forward unnormalised 3D DFT of a complex [nz][ny][nx] array (in place).
void oracle_fft3d(double *data, uint32_t nx, uint32_t ny, uint32_t nz) {
  fft3d(reinterpret_cast<cd *>(data), int(nx), int(ny), int(nz));
}

// NPP-semantics bilinear warp; dst must hold the prefill.
void oracle_warp(const double *src, double *dst, int width, int height, const double *coeffs) {
  double c[2][3] = {{coeffs[0], coeffs[1], coeffs[2]}, {coeffs[3], coeffs[4], coeffs[5]}};
  warp(src, dst, width, height, c);
}

// E-field direction E = R x for one E angle (radians) about a k vector, plus
// the base rotation angle (degrees are not used here).  Outputs R (row major).
void oracle_rotation(const float *k_in, int normalize_k, float eangle, float *R_out, float *base_out) {
  F3 k{k_in[0], k_in[1], k_in[2]};
  if (normalize_k) k = normalized(k);
  const FM rk = align({0.f, 0.f, 1.f}, k);
  const FM R = e_rotation(k, rk, eangle);
  std::memcpy(R_out, R.m, sizeof R.m);
  if (base_out) base_out[0] = base_angle(k, rk);
}

}  // extern "C"
