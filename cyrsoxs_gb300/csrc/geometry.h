// Host-side geometry of the scattering path: k-vector frames, the E-field
// rotation per angle, the per-angle image rotation and the detector warp.
//
// These decide discrete things downstream (which pixels are NaN, which Ewald
// plane is read), so they reproduce the reference's float arithmetic
// operation for operation:
//   Rotation.h:187-193 cross product, :272-315 vector-onto-vector rotation
//   (F G F^-1 with a double determinant), :326-338 Rodrigues, :422-465 base
//   angle scan, :474-484 per-angle E rotation, :499-516 affine from 3 points,
//   src/cudaMain.cu:612 E angle, :848-855 per-angle rotation coefficients,
//   :918-940 detector warp points.
// The bilinear warp's coordinate mapping follows nppiWarpAffine_32f_C1R
// (pinned bit-for-bit against the library on 49 probe images).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>

namespace cyr {

constexpr double kPi = 3.14159265358979323846;

struct Vec3f {
  float x, y, z;
};

struct Mat3f {
  float m[9];
  Mat3f() { std::memset(m, 0, sizeof m); }
  float &operator()(int i, int j) { return m[3 * i + j]; }
  float operator()(int i, int j) const { return m[3 * i + j]; }
  static Mat3f eye() {
    Mat3f r;
    r(0, 0) = r(1, 1) = r(2, 2) = 1.f;
    return r;
  }
};

inline bool near_equal(float a, float b) { return std::fabs(a - b) < 1e-6; }
inline float dot(Vec3f a, Vec3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec3f cross(Vec3f a, Vec3f b) { return {a.y * b.z - a.z * b.y, -(a.x * b.z - a.z * b.x), a.x * b.y - a.y * b.x}; }
inline float norm(Vec3f v) { return std::sqrt(dot(v, v)); }

inline Mat3f mul(const Mat3f &a, const Mat3f &b) {
  Mat3f r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) r.m[i * 3 + j] += a.m[i * 3 + k] * b.m[k * 3 + j];
  return r;
}

inline Vec3f apply(const Mat3f &a, Vec3f v) {
  return {a(0, 0) * v.x + a(0, 1) * v.y + a(0, 2) * v.z, a(1, 0) * v.x + a(1, 1) * v.y + a(1, 2) * v.z,
          a(2, 0) * v.x + a(2, 1) * v.y + a(2, 2) * v.z};
}

inline Mat3f inverse(const Mat3f &a) {
  const double det = a(0, 0) * (a(1, 1) * a(2, 2) - a(2, 1) * a(1, 2)) - a(0, 1) * (a(1, 0) * a(2, 2) - a(1, 2) * a(2, 0)) +
                     a(0, 2) * (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0));
  const float s = static_cast<float>(1. / det);
  Mat3f r;
  r(0, 0) = (a(1, 1) * a(2, 2) - a(2, 1) * a(1, 2)) * s;
  r(0, 1) = (a(0, 2) * a(2, 1) - a(0, 1) * a(2, 2)) * s;
  r(0, 2) = (a(0, 1) * a(1, 2) - a(0, 2) * a(1, 1)) * s;
  r(1, 0) = (a(1, 2) * a(2, 0) - a(1, 0) * a(2, 2)) * s;
  r(1, 1) = (a(0, 0) * a(2, 2) - a(0, 2) * a(2, 0)) * s;
  r(1, 2) = (a(1, 0) * a(0, 2) - a(0, 0) * a(1, 2)) * s;
  r(2, 0) = (a(1, 0) * a(2, 1) - a(2, 0) * a(1, 1)) * s;
  r(2, 1) = (a(2, 0) * a(0, 1) - a(0, 0) * a(2, 1)) * s;
  r(2, 2) = (a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1)) * s;
  return r;
}

// Rotation taking unit vector a onto unit vector b.
inline Mat3f rotation_between(Vec3f a, Vec3f b) {
  if (near_equal(a.x, b.x) && near_equal(a.y, b.y) && near_equal(a.z, b.z)) return Mat3f::eye();
  const float c = dot(a, b);
  const Vec3f ax = cross(a, b);
  const float s = norm(ax);
  Mat3f G;
  G(0, 0) = c;
  G(0, 1) = -s;
  G(1, 0) = s;
  G(1, 1) = c;
  G(2, 2) = 1.f;
  const Vec3f rej{b.x - c * a.x, b.y - c * a.y, b.z - c * a.z};
  const float nr = norm(rej);
  Mat3f F;
  F(0, 0) = a.x, F(1, 0) = a.y, F(2, 0) = a.z;
  F(0, 1) = rej.x / nr, F(1, 1) = rej.y / nr, F(2, 1) = rej.z / nr;
  F(0, 2) = -ax.x, F(1, 2) = -ax.y, F(2, 2) = -ax.z;
  return mul(F, mul(G, inverse(F)));
}

inline Vec3f rodrigues(Vec3f v, Vec3f axis, float angle) {
  const float c = std::cos(angle), s = std::sin(angle);
  const Vec3f cr = cross(axis, v);
  const float k = (1 - c) * dot(axis, v);
  return {c * v.x + s * cr.x + k * axis.x, c * v.y + s * cr.y + k * axis.y, c * v.z + s * cr.z + k * axis.z};
}

inline Vec3f unit(Vec3f v) {
  const float s = static_cast<float>(1. / norm(v));
  return {s * v.x, s * v.y, s * v.z};
}

// Frame of one k vector: R_k maps z onto k; base_angle makes E = x at 0 deg.
struct KFrame {
  Vec3f k;
  Mat3f rk;
  float base_angle;
};

inline KFrame make_kframe(Vec3f k) {
  KFrame f;
  f.k = k;
  f.rk = rotation_between({0.f, 0.f, 1.f}, k);
  constexpr uint32_t steps = 100000;
  constexpr float dtheta = static_cast<float>(kPi / (steps * 1.0));
  const Vec3f sx = apply(f.rk, {1.f, 0.f, 0.f});
  float best = std::numeric_limits<float>::infinity(), ang = 0.f;
  for (uint32_t i = 0; i < steps; ++i) {
    const float d = std::fabs(rodrigues(sx, k, i * dtheta).y);
    if (best > d) {
      best = d;
      ang = i * dtheta;
    }
  }
  f.base_angle = rodrigues(sx, k, ang).x > 0 ? ang : static_cast<float>(ang + kPi);
  return f;
}

// E-field rotation matrix R for an E angle in radians (E = R x).
inline Mat3f e_rotation(const KFrame &f, float angle) {
  const Vec3f sx = apply(f.rk, {1.f, 0.f, 0.f});
  return mul(rotation_between(sx, rodrigues(sx, f.k, angle)), f.rk);
}

// E angle (radians, float) of rotation step i.
inline float e_angle(const KFrame &f, float start, float inc, uint32_t i) {
  return static_cast<float>((f.base_angle + start + i * inc) * kPi / 180.0);
}

// Affine warp given as dst = C src; the per-angle rotation about the centre.
inline void rotation_coeffs(float eangle, uint32_t nx, uint32_t ny, double c[2][3]) {
  const double a = std::cos(eangle), b = std::sin(eangle);
  c[0][0] = a, c[0][1] = b, c[0][2] = static_cast<float>((1 - a) * nx / 2 - b * ny / 2.);
  c[1][0] = -b, c[1][1] = a, c[1][2] = static_cast<float>(b * nx / 2. + (1 - a) * ny / 2.);
}

inline void affine_from_points(const double s[3][2], const double d[3][2], double c[2][3]) {
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

// Detector warp for one k vector (identity for the default case).
inline void detector_coeffs(const Mat3f &det, const Mat3f &rk, uint32_t nx, uint32_t ny, double c[2][3]) {
  const double sp[3][2] = {{nx / 2., ny / 2.}, {nx * 0.5, ny * 1.0}, {nx * 1.0, ny * 0.5}};
  const double ctr[2] = {nx / 2., ny / 2.};
  const Mat3f m = mul(det, rk);
  double dp[3][2];
  for (int q = 0; q < 3; ++q) {
    const Vec3f s{static_cast<float>(sp[q][0] - ctr[0]), static_cast<float>(sp[q][1] - ctr[1]), 0.f};
    Vec3f d = apply(m, s);
    d.x = static_cast<float>(d.x + ctr[0]);
    d.y = static_cast<float>(d.y + ctr[1]);
    dp[q][0] = d.x, dp[q][1] = d.y;
  }
  affine_from_points(sp, dp, c);
}

// Inverse mapping used by the warp kernel: source = A dst, A in float with
// offsets formed in double from the rounded linear part.
struct WarpInverse {
  float a00, a01, a02, a10, a11, a12;
};

inline WarpInverse warp_inverse(const double c[2][3]) {
  const double det = c[0][0] * c[1][1] - c[0][1] * c[1][0];
  WarpInverse w;
  w.a00 = static_cast<float>(c[1][1] / det);
  w.a01 = static_cast<float>(-c[0][1] / det);
  w.a10 = static_cast<float>(-c[1][0] / det);
  w.a11 = static_cast<float>(c[0][0] / det);
  w.a02 = static_cast<float>(-(double(w.a00) * c[0][2] + double(w.a01) * c[1][2]));
  w.a12 = static_cast<float>(-(double(w.a10) * c[0][2] + double(w.a11) * c[1][2]));
  return w;
}

}  // namespace cyr
