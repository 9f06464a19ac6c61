// Device kernels of the GB300 scattering path.
//
// Data layout in HBM (all row-major, X fastest, as the reference's voxel
// index x + y*Nx + z*Nx*Ny, include/uniaxial.h:531-533):
//   voxels   float4 [M][V]               Voxel::s1 per material
//   spectra  float2 [nvol][V]            complex volumes (Nt columns or p)
//   images   float  [A][P]               per-angle Ewald intensity, P = Nx*Ny
//   avg      float  [P]                  angle average before the detector warp
//
// Every kernel is bounds-checked against the sizes it receives; no kernel
// waits on another block.
#pragma once

#include <cuda.h>  // CUtensorMap (the type only; encoded through the runtime's driver entry point)
#include <cuda_runtime.h>
#include <stdint.h>

namespace cyr {

constexpr int kMaxMaterials = 32;
constexpr int kMaxAngles = 4096;

// Complex add and subtract as packed FP32 pairs (add/sub.rn.f32x2, sm_100
// and later): one instruction performs both IEEE round-to-nearest operations,
// so each component is bit-identical to the scalar form, at half the
// instructions in the FFT butterflies.
__device__ __forceinline__ unsigned long long f2_pack(float2 v) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(v.x), "f"(v.y));
  return r;
}
__device__ __forceinline__ float2 f2_unpack(unsigned long long r) {
  float2 v;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
  return v;
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cfma(float s, float2 a, float2 acc) {
  return make_float2(fmaf(s, a.x, acc.x), fmaf(s, a.y, acc.y));
}

// ---------------------------------------------------------------------------
// 1. Dielectric tensor build.
//
// Per voxel, summed over materials, the six entries of
//   Nt = sum_m [ phi_a (A s s^T + B (|s|^2 I - s s^T)) + phi_ui C I ] / 4pi
// with A = n_par^2 - 1, B = n_perp^2 - 1, C = ((n_par + 2 n_perp)/3)^2 - 1
// formed in double on the host.  This is the reference's tensor
// (include/uniaxial.h:94-151 Euler, :218-274 vector) with the identity
// phi_a|s|^2 + phi_ui - phi = 0 applied exactly (Euler: |s| = 1 and
// phi = phi_a + phi_ui; vector: phi = phi_ui + |s|^2 by definition, :216),
// which removes the cancellation of n^2 ~ 1 against phi ~ 1 that limits the
// reference's FP32 build to ~1e-3.
// ---------------------------------------------------------------------------
struct MaterialConsts {
  float2 A[kMaxMaterials];  // (n_par^2 - 1) / 4pi
  float2 B[kMaxMaterials];  // (n_perp^2 - 1) / 4pi
  float2 C[kMaxMaterials];  // (((n_par + 2 n_perp)/3)^2 - 1) / 4pi
  float2 D[kMaxMaterials];  // (n_par^2 - n_perp^2) / 4pi
};

struct BuildParams {
  const float4 *vox;
  uint32_t nx, ny, nz, nmat;
  size_t nvox;
  uint32_t morphology;  // 0 Euler, 1 vector
  uint32_t mode;        // 0: tensor entries; 1: p = R-frame polarization
  uint32_t nvol;        // mode 0: entries xx xy xz yy yz [zz] written in this order
  const float2 *mean;   // [6] volume mean of each windowed entry (null: none subtracted)
  const float4 *conv;   // Euler morphology converted to (sqrt(phi_a) s, phi_ui) per material, or null
  const unsigned *neg;  // set when some phi_a < 0 (the conversion is then not used)
  float E[3];           // mode 1: E = R x
  float Rm[9];          // mode 1: R (row major), for the MATERIAL frame
  uint32_t material_frame;
  const float *hann_x, *hann_y, *hann_z;  // null when no windowing
  float2 *out;          // [nvol][V]
};

// Direction and fractions of one material at one voxel.
template <int MORPH>
__device__ __forceinline__ void director(float4 s, float &sx, float &sy, float &sz, float &pa, float &pui) {
  if (MORPH == 0) {  // Euler: s1 = (S, theta, psi, Vfrac), uniaxial.h:82-92
    float st, ct, sp, cp;
    sincosf(s.y, &st, &ct);
    sincosf(s.z, &sp, &cp);
    sx = cp * st;
    sy = sp * st;
    sz = ct;
    pa = s.w * s.x;
    pui = s.w - pa;
  } else {  // vector: s1 = (sx, sy, sz, phi_unaligned), uniaxial.h:207-216
    sx = s.x, sy = s.y, sz = s.z;
    pa = 1.f;
    pui = s.w;
  }
}

// Tensor entries of one voxel.  With CONV the morphology has been converted
// to the vector form u = sqrt(phi_a) s, phi_ui (phi_a s_i s_j = u_i u_j),
// which needs no trigonometry per energy.
// `base` points at material 0 of the voxel, material m at base + m * mstride
// (global memory, or a tile staged in shared memory).
template <int MORPH, bool CONV>
__device__ __forceinline__ void nt_entries_at(const BuildParams &p, const MaterialConsts &mc, const float4 *base,
                                              size_t mstride, float2 nt[6]) {
#pragma unroll
  for (int q = 0; q < 6; ++q) nt[q] = make_float2(0.f, 0.f);
  for (uint32_t m0 = 0; m0 < p.nmat; m0 += 4) {
    float4 sv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u)  // issue the loads of up to 4 materials before using them
      if (m0 + u < p.nmat) sv[u] = base[(m0 + u) * mstride];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (m0 + u >= p.nmat) break;
      const uint32_t m = m0 + u;
      float sx, sy, sz, pa, pui;
      director<CONV ? 1 : MORPH>(sv[u], sx, sy, sz, pa, pui);
      const float xx = sx * sx, yy = sy * sy, zz = sz * sz;
      const float2 A = mc.A[m], B = mc.B[m], C = mc.C[m], D = mc.D[m];
      // diagonal: phi_a (A s_i^2 + B (|s|^2 - s_i^2)) + phi_ui C, with |s|^2 - s_i^2 as the reference sums it
      const float ax = pa * xx, ay = pa * yy, az = pa * zz;
      const float bx = pa * (yy + zz), by = pa * (xx + zz), bz = pa * (xx + yy);
      nt[0].x += ax * A.x + bx * B.x + pui * C.x;
      nt[0].y += ax * A.y + bx * B.y + pui * C.y;
      nt[3].x += ay * A.x + by * B.x + pui * C.x;
      nt[3].y += ay * A.y + by * B.y + pui * C.y;
      nt[5].x += az * A.x + bz * B.x + pui * C.x;
      nt[5].y += az * A.y + bz * B.y + pui * C.y;
      const float pxy = pa * sx * sy, pxz = pa * sx * sz, pyz = pa * sy * sz;
      nt[1] = cfma(pxy, D, nt[1]);
      nt[2] = cfma(pxz, D, nt[2]);
      nt[4] = cfma(pyz, D, nt[4]);
    }
  }
}

template <int MORPH, bool CONV>
__device__ __forceinline__ void nt_entries(const BuildParams &p, const MaterialConsts &mc, size_t i, float2 nt[6]) {
  nt_entries_at<MORPH, CONV>(p, mc, (CONV ? p.conv : p.vox) + i, p.nvox, nt);
}

// Volume moments of the morphology, per material, in double:
// <w phi_a s_x^2>, <w phi_a s_y^2>, <w phi_a s_z^2>, <w phi_a s_x s_y>,
// <w phi_a s_x s_z>, <w phi_a s_y s_z>, <w phi_ui> (sums; w = window or 1).
// With the per-energy constants they give the mean of every tensor entry.
// Subtracting a constant before the FFT changes only frequency bin 0, which
// the path always replaces by the mean of its neighbours (src/cudaMain.cu:
// 123-176); removing it keeps the FP32 FFT's rounding floor proportional to
// the fluctuations instead of to the (~5x larger) mean.
constexpr int kMoments = 7;
struct MomentParams {
  const float4 *vox;
  const float4 *const *vox_g;  // request group (blockIdx.z = request): its morphologies, or null
  uint32_t nx, ny, nz, nmat;
  size_t nvox;
  const float *hann_x, *hann_y, *hann_z;
  double *out;      // [nmat][kMoments], accumulated
  float4 *conv;     // Euler only: (sqrt(phi_a) s, phi_ui) per material and voxel, or null
  unsigned *neg;    // set when some phi_a < 0
  uint32_t zstep;   // sample every zstep-th z plane (1: all; must be 1 with conv)
};

template <int MORPH>
__global__ void __launch_bounds__(256) k_moments(MomentParams p) {
  __shared__ double red[8][kMoments];
  const uint32_t m = blockIdx.y;
  if (p.vox_g) {  // a request group: request blockIdx.z's morphology and moments
    p.vox = p.vox_g[blockIdx.z];
    p.out += size_t(blockIdx.z) * p.nmat * kMoments;
  }
  // per-thread sums in float (a few hundred terms; only an approximate mean is
  // needed), block and grid reduction in double
  float acc[kMoments];
#pragma unroll
  for (int q = 0; q < kMoments; ++q) acc[q] = 0.f;
  // samples: every pixel of the planes z = 0, zstep, 2 zstep, ...; the
  // thread's (sampled plane, pixel) position advances by the grid stride
  // without an index division per sample
  const size_t plane = size_t(p.nx) * p.ny, stride = size_t(gridDim.x) * blockDim.x;
  const uint32_t nzs = (p.nz + p.zstep - 1) / p.zstep;
  const size_t s0 = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  uint32_t zi = uint32_t(s0 / plane);
  size_t pix = s0 - size_t(zi) * plane;
  for (; zi < nzs; pix += stride) {
    while (pix >= plane) pix -= plane, ++zi;
    if (zi >= nzs) break;
    const size_t i = size_t(zi) * p.zstep * plane + pix;
    float sx, sy, sz, pa, pui;
    director<MORPH>(__ldg(&p.vox[m * p.nvox + i]), sx, sy, sz, pa, pui);
    if (MORPH == 0 && p.conv) {
      if (pa < 0.f) atomicOr(p.neg, 1u);
      const float r = sqrtf(fmaxf(pa, 0.f));
      p.conv[m * p.nvox + i] = make_float4(r * sx, r * sy, r * sz, pui);
    }
    float w = 1.f;
    if (p.hann_x) {
      const uint32_t x = uint32_t(pix) % p.nx, y = uint32_t(pix) / p.nx, z = zi * p.zstep;
      w = p.hann_x[x] * p.hann_y[y] * p.hann_z[z];
    }
    const float wa = w * pa;
    acc[0] += wa * sx * sx;
    acc[1] += wa * sy * sy;
    acc[2] += wa * sz * sz;
    acc[3] += wa * sx * sy;
    acc[4] += wa * sx * sz;
    acc[5] += wa * sy * sz;
    acc[6] += w * pui;
  }
#pragma unroll
  for (int q = 0; q < kMoments; ++q) {
    double v = double(acc[q]);
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < kMoments) {
    double v = 0.0;
    for (int wi = 0; wi < int(blockDim.x >> 5); ++wi) v += red[wi][threadIdx.x];
    atomicAdd(&p.out[m * kMoments + threadIdx.x], v);
  }
}

// Mean of each windowed tensor entry for every energy: out[e][6] (xx xy xz yy yz zz).
__global__ void k_entry_means(const double *__restrict__ mom, uint32_t nmat, size_t nvox,
                              const MaterialConsts *__restrict__ mcs, uint32_t ne, float2 *__restrict__ out) {
  for (uint32_t e = threadIdx.x; e < ne; e += blockDim.x) {
    double r[6][2] = {};
    for (uint32_t m = 0; m < nmat; ++m) {
      const double *M = mom + m * kMoments;
      const MaterialConsts &c = mcs[e];
      const double A[2] = {c.A[m].x, c.A[m].y}, B[2] = {c.B[m].x, c.B[m].y};
      const double C[2] = {c.C[m].x, c.C[m].y}, D[2] = {c.D[m].x, c.D[m].y};
      for (int k = 0; k < 2; ++k) {
        r[0][k] += A[k] * M[0] + B[k] * (M[1] + M[2]) + C[k] * M[6];
        r[3][k] += A[k] * M[1] + B[k] * (M[0] + M[2]) + C[k] * M[6];
        r[5][k] += A[k] * M[2] + B[k] * (M[0] + M[1]) + C[k] * M[6];
        r[1][k] += D[k] * M[3];
        r[2][k] += D[k] * M[4];
        r[4][k] += D[k] * M[5];
      }
    }
    for (int q = 0; q < 6; ++q)
      out[e * 6 + q] = make_float2(float(r[q][0] / double(nvox)), float(r[q][1] / double(nvox)));
  }
}

// The values one voxel contributes to the FFT input: mode 0 the windowed tensor
// entries xx xy xz yy yz [zz] (nvol of them), mode 1 the polarization
// p = Nt E (uniaxial.h:106-151), rotated by R^T in the MATERIAL frame
// (:163-165); the volume mean is subtracted when p.mean is set.
__device__ __forceinline__ void values_from_nt(const BuildParams &p, float2 nt[6], uint32_t x, uint32_t y, uint32_t z,
                                               float2 out[6]);

template <int MORPH, bool CONV>
__device__ __forceinline__ void voxel_values(const BuildParams &p, const MaterialConsts &mc, size_t i, uint32_t x,
                                             uint32_t y, uint32_t z, float2 out[6]) {
  float2 nt[6];
  nt_entries<MORPH, CONV>(p, mc, i, nt);
  values_from_nt(p, nt, x, y, z, out);
}

// Window, mean removal and (mode 1) the E / R^T maps applied to a voxel's tensor.
__device__ __forceinline__ void values_from_nt(const BuildParams &p, float2 nt[6], uint32_t x, uint32_t y, uint32_t z,
                                               float2 out[6]) {
  const float w = p.hann_x ? p.hann_x[x] * p.hann_y[y] * p.hann_z[z] : 1.f;
  if (p.mode == 0) {
#pragma unroll
    for (int v = 0; v < 6; ++v) {
      out[v] = cscale(nt[v], w);
      if (p.mean) out[v] = csub(out[v], p.mean[v]);
    }
    return;
  }
  const float e0 = p.E[0], e1 = p.E[1], e2 = p.E[2];
  float2 q[3];
#pragma unroll
  for (int pass = 0; pass < 2; ++pass) {
    // pass 0: this voxel; pass 1 (only with means): the mean tensor, same linear map
    float2 t[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) t[c] = pass == 0 ? cscale(nt[c], w) : (p.mean ? p.mean[c] : make_float2(0.f, 0.f));
    float2 r3[3];
    r3[0] = cadd(cadd(cscale(t[0], e0), cscale(t[1], e1)), cscale(t[2], e2));
    r3[1] = cadd(cadd(cscale(t[1], e0), cscale(t[3], e1)), cscale(t[4], e2));
    r3[2] = cadd(cadd(cscale(t[2], e0), cscale(t[4], e1)), cscale(t[5], e2));
    if (p.material_frame) {
      float2 r[3];
#pragma unroll
      for (int a = 0; a < 3; ++a)
        r[a] = cadd(cadd(cscale(r3[0], p.Rm[0 * 3 + a]), cscale(r3[1], p.Rm[1 * 3 + a])), cscale(r3[2], p.Rm[2 * 3 + a]));
      r3[0] = r[0], r3[1] = r[1], r3[2] = r[2];
    }
    if (pass == 0) {
      q[0] = r3[0], q[1] = r3[1], q[2] = r3[2];
    } else {
      q[0] = csub(q[0], r3[0]), q[1] = csub(q[1], r3[1]), q[2] = csub(q[2], r3[2]);
    }
    if (!p.mean) break;
  }
  out[0] = q[0], out[1] = q[1], out[2] = q[2];
  out[3] = out[4] = out[5] = make_float2(0.f, 0.f);
}

__device__ __forceinline__ void load_consts(MaterialConsts &dst, const MaterialConsts *src) {
  const float *s = reinterpret_cast<const float *>(src);
  float *d = reinterpret_cast<float *>(&dst);
  for (int t = threadIdx.x; t < int(sizeof(MaterialConsts) / 4); t += blockDim.x) d[t] = s[t];
}

// CONV selects the converted (trigonometry-free) morphology; for Euler input
// both instantiations are launched and the one that does not match the
// device-side flag returns at once.
__device__ __forceinline__ bool conv_selected(const BuildParams &p) { return p.conv && *p.neg == 0u; }

template <int MORPH, bool CONV>
__global__ void __launch_bounds__(256) k_build(BuildParams p, const MaterialConsts *__restrict__ mcp) {
  if (MORPH == 0 && conv_selected(p) != CONV) return;
  __shared__ MaterialConsts mc;
  load_consts(mc, mcp);
  __syncthreads();
  const size_t stride = size_t(gridDim.x) * blockDim.x;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < p.nvox; i += stride) {
    const uint32_t x = uint32_t(i % p.nx), y = uint32_t((i / p.nx) % p.ny), z = uint32_t(i / (size_t(p.nx) * p.ny));
    float2 v[6];
    voxel_values<MORPH, CONV>(p, mc, i, x, y, z, v);
#pragma unroll
    for (int c = 0; c < 6; ++c)
      if (uint32_t(c) < p.nvol) p.out[c * p.nvox + i] = v[c];
  }
}

// ---------------------------------------------------------------------------
// 2. Forward FFT along one axis: shared-memory Stockham autosort, mixed radix
// {8, 4, 2, 3, 5, 7}, twiddles generated in FP64 on the host (W_N^m table).
// A block transforms TX lines at once, interleaved in shared memory as
// [n][TX+1] so that lanes of a warp touch consecutive words.  The X pass
// loads TX consecutive rows; the Y and Z passes load TX consecutive
// x-columns, so every global access is a run of TX*8 contiguous bytes or more.
// Two buffers (ping-pong) make each stage one read and one write per element.
// ---------------------------------------------------------------------------
struct FftAxis {
  uint32_t n;            // line length
  uint32_t log2n;        // log2(n) when n is a power of two, else 0
  uint32_t nstages;
  uint64_t radix_code;   // radix of stage s in bits [4s, 4s+4)
  const float2 *tw;      // W_n^m, m in [0, n)
};

__device__ __forceinline__ void dft2(float2 *v) {
  const float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }  // a * (-i)
__device__ __forceinline__ void dft4(float2 &v0, float2 &v1, float2 &v2, float2 &v3) {
  const float2 t0 = cadd(v0, v2), t1 = csub(v0, v2), t2 = cadd(v1, v3), t3 = mul_mi(csub(v1, v3));
  v0 = cadd(t0, t2);
  v2 = csub(t0, t2);
  v1 = cadd(t1, t3);
  v3 = csub(t1, t3);
}
__device__ __forceinline__ void dft8(float2 *v) {
  float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4(e0, e1, e2, e3);
  dft4(o0, o1, o2, o3);
  const float h = 0.70710678118654752440f;
  o1 = make_float2(h * (o1.x + o1.y), h * (o1.y - o1.x));     // * W8^1 = (1 - i)/sqrt2
  o2 = mul_mi(o2);                                            // * W8^2 = -i
  o3 = make_float2(h * (o3.y - o3.x), -h * (o3.x + o3.y));    // * W8^3 = -(1 + i)/sqrt2
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  v[1] = cadd(e1, o1);
  v[5] = csub(e1, o1);
  v[2] = cadd(e2, o2);
  v[6] = csub(e2, o2);
  v[3] = cadd(e3, o3);
  v[7] = csub(e3, o3);
}
// Odd prime radices: direct DFT with cos/sin(2 pi m / R) constants.
template <int R>
__device__ __forceinline__ void dft_odd(float2 *v) {
  float cs[R], sn[R];
  if (R == 3) {
    cs[0] = 1.f, sn[0] = 0.f, cs[1] = -0.5f, sn[1] = 0.86602540378443864676f, cs[2] = -0.5f, sn[2] = -0.86602540378443864676f;
  } else if (R == 5) {
    const float c1 = 0.30901699437494742410f, s1 = 0.95105651629515357212f;
    const float c2 = -0.80901699437494742410f, s2 = 0.58778525229247312917f;
    cs[0] = 1.f, sn[0] = 0.f, cs[1] = c1, sn[1] = s1, cs[2] = c2, sn[2] = s2, cs[3] = c2, sn[3] = -s2, cs[4] = c1,
    sn[4] = -s1;
  } else {
    const float c1 = 0.62348980185873353053f, s1 = 0.78183148246802980871f;
    const float c2 = -0.22252093395631440429f, s2 = 0.97492791218182360702f;
    const float c3 = -0.90096886790241912624f, s3 = 0.43388373911755812048f;
    cs[0] = 1.f, sn[0] = 0.f, cs[1] = c1, sn[1] = s1, cs[2] = c2, sn[2] = s2, cs[3] = c3, sn[3] = s3;
    cs[4] = c3, sn[4] = -s3, cs[5] = c2, sn[5] = -s2, cs[6] = c1, sn[6] = -s1;
  }
  float2 out[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    float2 acc = v[0];
#pragma unroll
    for (int j = 1; j < R; ++j) {
      const int m = (j * q) % R;  // W_R^{jq} = cos - i sin
      acc.x += v[j].x * cs[m] + v[j].y * sn[m];
      acc.y += v[j].y * cs[m] - v[j].x * sn[m];
    }
    out[q] = acc;
  }
#pragma unroll
  for (int q = 0; q < R; ++q) v[q] = out[q];
}

// One Stockham stage of radix R over all lines of the block.  The block holds
// `nv` groups of `lines` interleaved lines; element i of line l in group v
// lives at (v * n + i) * S + l.
template <int R>
__device__ __forceinline__ void stockham_stage(const float2 *__restrict__ src, float2 *__restrict__ dst, uint32_t n,
                                               uint32_t ns, uint32_t lines, uint32_t nv, uint32_t S,
                                               const float2 *__restrict__ tw, bool pow2, uint32_t lg_lines,
                                               uint32_t lg_m, uint32_t lg_ns) {
  const uint32_t m = n / R;               // butterflies per line
  const uint32_t twstep = n / (ns * R);   // W_{ns R}^{k r} = W_n^{k r twstep}
  const uint32_t jobs = m * lines * nv;
  const uint32_t mS = m * S, nsS = ns * S;
  for (uint32_t job = threadIdx.x; job < jobs; job += blockDim.x) {
    const uint32_t l = job & (lines - 1), rest = job >> lg_lines;  // lines is a power of two
    uint32_t j, v, k, q;
    if (pow2) {
      j = rest & (m - 1), v = rest >> lg_m, k = j & (ns - 1), q = j >> lg_ns;
    } else {
      j = rest % m, v = rest / m, k = j % ns, q = j / ns;
    }
    const uint32_t vb = v * n;  // shared-memory offsets fit in 32 bits
    const uint32_t in0 = (vb + j) * S + l;
    float2 w[R];
#pragma unroll
    for (int r = 0; r < R; ++r) w[r] = src[in0 + r * mS];
    if (ns > 1) {
      const uint32_t t1 = k * twstep;
#pragma unroll
      for (int r = 1; r < R; ++r) w[r] = cmul(w[r], tw[t1 * r]);
    }
    if (R == 2) dft2(w);
    if (R == 4) dft4(w[0], w[1], w[2], w[3]);
    if (R == 8) dft8(w);
    if (R == 3 || R == 5 || R == 7) dft_odd<(R == 2 || R == 4 || R == 8) ? 3 : R>(w);
    const uint32_t out0 = (vb + q * ns * R + k) * S + l;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[out0 + r * nsS] = w[r];
  }
}

// Copies the twiddle table W_n^m (m < n) into shared memory.
__device__ __forceinline__ void stage_twiddles(float2 *dst, const float2 *__restrict__ src, uint32_t n) {
  for (uint32_t t = threadIdx.x; t < n; t += blockDim.x) dst[t] = __ldg(&src[t]);
}

// Runs all stages; returns the buffer holding the result.  `lines` must be a
// power of two.
__device__ __forceinline__ float2 *stockham(float2 *a, float2 *b, const FftAxis &ax, const float2 *tw,
                                            uint32_t lines, uint32_t S, uint32_t nv = 1) {
  const bool pow2 = ax.log2n != 0;
  const uint32_t lg_lines = 31 - __clz(lines);
  uint32_t ns = 1, lg_ns = 0;
  for (uint32_t s = 0; s < ax.nstages; ++s) {
    const uint32_t R = uint32_t(ax.radix_code >> (4 * s)) & 15u;
    const uint32_t lg_r = R == 8 ? 3 : R == 4 ? 2 : 1;
    const uint32_t lg_m = pow2 ? ax.log2n - lg_r : 0;
    switch (R) {
      case 8: stockham_stage<8>(a, b, ax.n, ns, lines, nv, S, tw, pow2, lg_lines, lg_m, lg_ns); break;
      case 4: stockham_stage<4>(a, b, ax.n, ns, lines, nv, S, tw, pow2, lg_lines, lg_m, lg_ns); break;
      case 2: stockham_stage<2>(a, b, ax.n, ns, lines, nv, S, tw, pow2, lg_lines, lg_m, lg_ns); break;
      case 3: stockham_stage<3>(a, b, ax.n, ns, lines, nv, S, tw, false, lg_lines, 0, 0); break;
      case 5: stockham_stage<5>(a, b, ax.n, ns, lines, nv, S, tw, false, lg_lines, 0, 0); break;
      default: stockham_stage<7>(a, b, ax.n, ns, lines, nv, S, tw, false, lg_lines, 0, 0); break;
    }
    __syncthreads();
    float2 *t = a;
    a = b;
    b = t;
    ns *= R;
    lg_ns += lg_r;
  }
  return a;
}

// Asynchronous global -> shared copies (cp.async, 8 bytes each): every load of
// a tile is in flight at once instead of one per thread per loop iteration.
__device__ __forceinline__ void cp_async8(void *smem_dst, const void *gmem_src) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src) : "memory");
}

// AXIS 0: lines along x (rows).  AXIS 1: along y.  AXIS 2: along z.
// Grid: x = tiles, y = volume.  TX lines per tile (TX * n ~ 4096 elements,
// two 32 KB buffers, 3 blocks of 512 threads per SM).
constexpr int kFftThreads = 512;
struct FftPassParams {
  float2 *data;
  uint32_t nx, ny, nz;
  size_t nvox;
  uint32_t tx;  // lines per block
  FftAxis ax;
};

template <int AXIS>
__global__ void __launch_bounds__(kFftThreads, 3) k_fft_pass(FftPassParams p) {
  extern __shared__ float2 smem[];
  const uint32_t n = p.ax.n, TX = p.tx, S = TX + 1;
  float2 *bufa = smem, *bufb = smem + n * S, *tws = smem + 2 * n * S;
  // Tile geometry: line l starts at tile + l * lstep; element i at + i * estep
  // (offsets inside one volume fit in 32 bits).
  size_t base;
  uint32_t valid, lstep, estep;
  if (AXIS == 0) {
    const uint32_t rows = p.ny * p.nz;
    const uint32_t r0 = blockIdx.x * TX;
    base = size_t(r0) * p.nx;
    valid = min(TX, rows - r0);
    lstep = p.nx;
    estep = 1;
  } else {
    const uint32_t nxt = (p.nx + TX - 1) / TX;
    const uint32_t xt = blockIdx.x % nxt, other = blockIdx.x / nxt;
    const uint32_t x0 = xt * TX;
    valid = min(TX, p.nx - x0);
    lstep = 1;
    if (AXIS == 1) {
      base = size_t(other) * p.nx * p.ny + x0;  // other = z
      estep = p.nx;
    } else {
      base = size_t(other) * p.nx + x0;  // other = y
      estep = p.nx * p.ny;
    }
  }
  float2 *tile = p.data + size_t(blockIdx.y) * p.nvox + base;
  const uint32_t total = n * TX;
  for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
    uint32_t l, i;
    if (AXIS == 0) {
      l = t / n, i = t % n;  // consecutive threads walk along a row
    } else {
      l = t % TX, i = t / TX;  // consecutive threads walk across the tile's columns
    }
    float2 *dst = &bufa[i * S + l];
    if (l < valid)
      cp_async8(dst, &tile[l * lstep + i * estep]);
    else
      *dst = make_float2(0.f, 0.f);
  }
  stage_twiddles(tws, p.ax.tw, n);
  cp_async_wait_all();
  __syncthreads();
  const float2 *res = stockham(bufa, bufb, p.ax, tws, TX, S);
  for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
    uint32_t l, i;
    if (AXIS == 0) {
      l = t / n, i = t % n;
    } else {
      l = t % TX, i = t / TX;
    }
    if (l < valid) tile[l * lstep + i * estep] = res[i * S + l];
  }
}

// ---------------------------------------------------------------------------
// Bluestein (chirp-z) transform, for line lengths N with a prime factor above 7
// (cuFFT's cufftPlan3d accepts every size, src/cudaMain.cu:479-482).
//
// With c_j = exp(-i pi j^2 / N), jk = (j^2 + k^2 - (k - j)^2) / 2 gives
//   X_k = c_k sum_j (x_j c_j) conj(c_{k-j}),
// a circular convolution of length M >= 2N - 1 (M 7-smooth), evaluated as
// FFT_M -> product with the table bhat = FFT_M(b) / M, where b holds
// conj(c_m) at m and M - m -> a second FFT_M of the conjugate, since the
// inverse transform is conj(FFT(conj(y))) / M.  Chirp and table are formed in
// double on the host (j^2 reduced mod 2N in integers) and rounded to float.
// The lines of a pass are processed in chunks of `nlines` padded lines held
// in `work`: [nlines][M] for x lines (the padded FFT is a row pass), [M][nlines]
// for y and z lines (a column pass), so every gather, product and scatter
// reads and writes contiguous memory.
// ---------------------------------------------------------------------------
// T = float2 for the FP32 engine, double2 for the FP64 pipeline (its tables in double).
template <class T>
struct BlueParamsT {
  T *data;                // the volumes being transformed
  T *work;                // x lines: [nlines][m]; y and z lines: [m][nlines] (lines fastest)
  const T *chirp;         // c_j, j < n
  const T *bhat;          // FFT_m(b) / m
  uint32_t nx, ny, nz;    // volume dimensions (nz: the planes this call covers)
  size_t vstride;         // elements between volumes
  uint32_t n, m;          // line length, padded length
  uint64_t line0;         // first line of this chunk
  uint32_t nlines;        // lines in this chunk
  uint32_t lines_per_vol; // x pass: ny nz; y pass: nx nz; z pass: nx ny
};
using BlueParams = BlueParamsT<float2>;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Offset of line `line` and the stride between its elements.
template <int AXIS, class P>
__device__ __forceinline__ size_t blue_line(const P &p, uint64_t line, size_t &estep) {
  const uint64_t v = line / p.lines_per_vol;
  const uint32_t r = uint32_t(line % p.lines_per_vol);
  size_t base = v * p.vstride;
  if (AXIS == 0) {
    base += size_t(r) * p.nx;
    estep = 1;
  } else if (AXIS == 1) {
    base += size_t(r / p.nx) * p.nx * p.ny + r % p.nx;
    estep = p.nx;
  } else {
    base += size_t(r / p.nx) * p.nx + r % p.nx;
    estep = size_t(p.nx) * p.ny;
  }
  return base;
}

// work = x_j c_j (j < n), 0 (n <= j < m).  Thread t takes element t of the
// work buffer, so its stores are contiguous; for y and z lines consecutive
// lines are consecutive x, so the volume reads are contiguous too.
template <int AXIS, class T = float2>
__global__ void k_blue_gather(BlueParamsT<T> p) {
  const size_t total = size_t(p.nlines) * p.m;
  for (size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x; t < total; t += size_t(gridDim.x) * blockDim.x) {
    uint32_t l, j;
    if (AXIS == 0) {
      l = uint32_t(t / p.m), j = uint32_t(t % p.m);
    } else {
      l = uint32_t(t % p.nlines), j = uint32_t(t / p.nlines);
    }
    T v{};
    if (j < p.n) {
      size_t es;
      const size_t b = blue_line<AXIS>(p, p.line0 + l, es);
      v = cmul(p.data[b + j * es], p.chirp[j]);
    }
    p.work[t] = v;
  }
}

// work = conj(work * bhat): the product of the transforms, conjugated for the inverse
template <int AXIS, class T = float2>
__global__ void k_blue_mul(BlueParamsT<T> p) {
  const size_t total = size_t(p.nlines) * p.m;
  for (size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x; t < total; t += size_t(gridDim.x) * blockDim.x) {
    const T w = cmul(p.work[t], p.bhat[AXIS == 0 ? t % p.m : t / p.nlines]);
    p.work[t] = T{w.x, -w.y};
  }
}

// x_k = c_k conj(work element k of line l), k < n
template <int AXIS, class T = float2>
__global__ void k_blue_scatter(BlueParamsT<T> p) {
  const size_t total = size_t(p.nlines) * p.n;
  for (size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x; t < total; t += size_t(gridDim.x) * blockDim.x) {
    uint32_t l, k;
    size_t wi;
    if (AXIS == 0) {
      l = uint32_t(t / p.n), k = uint32_t(t % p.n);
      wi = size_t(l) * p.m + k;
    } else {
      l = uint32_t(t % p.nlines), k = uint32_t(t / p.nlines);
      wi = t;  // element k of line l at k nlines + l
    }
    const T w = p.work[wi];
    size_t es;
    const size_t b = blue_line<AXIS>(p, p.line0 + l, es);
    p.data[b + k * es] = cmul(p.chirp[k], T{w.x, -w.y});
  }
}

// ---------------------------------------------------------------------------
// Warp-level FFT for power-of-two lengths N = 32 V (V = 4, 8, 16, 32).
//
// One warp owns one line.  Lane t holds x[t + 32 i] in v[i] (natural order)
// on entry and X[t + 32 i] on exit.  Each Stockham stage of radix R <= V runs
// V / R butterflies per lane on registers; between stages the lanes exchange
// through the warp's own line in shared memory (swizzled, swz: free of bank
// conflicts for every access of the plan), so only __syncwarp is needed.  The last stage's outputs land in natural order in
// registers.  Twiddles W_N^m (generated in FP64) are staged per stage in the
// order the lanes read them (warp_twiddles).
// ---------------------------------------------------------------------------
// Shared-memory slot of element p of a line: the 8-byte bank (the low 4 bits)
// is XORed with a GF(2)-linear function of the higher bits.  The masks were
// found by an exhaustive check of every access of the V = 4, 8, 16 plans
// (contiguous reads, each stage's strided stores) and of the TX-column tile
// copies (TX = 2..16, line_stride below): no half-warp access puts two lanes
// on one bank.  A bijection on [0, N), so lines need no padding.
__host__ __device__ constexpr uint32_t swz_mask(uint32_t h) {  // h = p >> 4
  return ((h & 1u) ? 10u : 0u) ^ ((h & 2u) ? 15u : 0u) ^ ((h & 4u) ? 12u : 0u) ^ ((h & 8u) ? 3u : 0u) ^
         ((h & 16u) ? 12u : 0u);
}
__device__ __forceinline__ uint32_t swz(uint32_t p) { return p ^ swz_mask(p >> 4); }
// swz(t + 32 i) for t < 32 given tx = swz(t): swz_mask is linear over GF(2)
// and t, 32 i occupy disjoint bits, so swz(t | 32 i) = swz(t) ^ 32 i ^
// swz_mask(2 i); with i a compile-time constant that is a single XOR.
__device__ __forceinline__ uint32_t swz_at(uint32_t tx, uint32_t i) { return tx ^ (32u * i) ^ swz_mask(2u * i); }
// Stride between the lines of TX interleaved columns: congruent to 16 / TX
// (1 for TX >= 16) modulo 16, so a half-warp touching TX columns x (16 / TX)
// consecutive positions hits 16 distinct 8-byte banks.
__host__ __device__ constexpr uint32_t line_stride(uint32_t n, uint32_t tx) {
  return ((n + 15u) & ~15u) + (tx >= 16 ? 1u : 16u / tx);
}

template <int V>
struct WarpPlan {
  static constexpr int N = 32 * V;
  static constexpr int LOG2N = V == 4 ? 7 : V == 8 ? 8 : V == 16 ? 9 : 10;
  // radices: as many 8s as V allows, then one 4 or 2 for the remainder
  static constexpr int MAXR = V >= 8 ? 8 : V;
  static constexpr int LOGMAXR = MAXR == 8 ? 3 : MAXR == 4 ? 2 : 1;
  static constexpr int NFULL = LOG2N / LOGMAXR;
  static constexpr int REM = LOG2N - NFULL * LOGMAXR;  // 0, 1 or 2
  static constexpr int NSTAGES = NFULL + (REM ? 1 : 0);
  __host__ __device__ static constexpr int radix(int s) { return s < NFULL ? MAXR : (REM == 2 ? 4 : 2); }
};

// Shared twiddle tables of the warp FFT: stage s > 0 (NS > 1, radix R) holds
// W_N^(k r N / (NS R)) at [NS - R0 + k (R - 1) + r - 1] for k < NS, 1 <= r < R
// (N - R0 entries in all).  The lanes of a half-warp read 16 consecutive k,
// addresses an odd R - 1 apart: 16 distinct banks, where the strided table
// W_N^(k r TWS) put up to 8 lanes on one bank.
template <int V>
__device__ __forceinline__ void warp_twiddles(float2 *dst, const float2 *__restrict__ tw_n) {
  using P = WarpPlan<V>;
  constexpr uint32_t N = P::N, R0 = P::radix(0);
  for (uint32_t t = threadIdx.x; t < N - R0; t += blockDim.x) {
    uint32_t ns = R0, base = 0;
#pragma unroll
    for (int s = 1; s < P::NSTAGES; ++s) {
      const uint32_t R = P::radix(s), cnt = ns * (R - 1);
      if (t >= base && t < base + cnt) {
        const uint32_t u = t - base, k = u / (R - 1), r = u % (R - 1) + 1;
        dst[t] = __ldg(&tw_n[k * r * (N / (ns * R))]);
      }
      base += cnt;
      ns *= R;
    }
  }
}

template <int V, int R, int NS, bool LAST>
__device__ __forceinline__ void warp_stage(float2 (&v)[V], float2 *line, const float2 *__restrict__ tw,
                                           uint32_t lane) {
  constexpr int B = V / R;                          // butterflies per lane
  constexpr int TWOFF = NS > 1 ? NS - WarpPlan<V>::radix(0) : 0;  // this stage's table (warp_twiddles)
#pragma unroll
  for (int q = 0; q < B; ++q) {
    const uint32_t j = lane + 32 * q;
    const uint32_t k = j & (NS - 1);
    float2 w[R];
#pragma unroll
    for (int r = 0; r < R; ++r) w[r] = v[q + r * B];
    if (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) w[r] = cmul(w[r], tw[TWOFF + k * (R - 1) + r - 1]);
    }
    if (R == 2) dft2(w);
    if (R == 4) dft4(w[0], w[1], w[2], w[3]);
    if (R == 8) dft8(w);
    if (LAST) {
#pragma unroll
      for (int r = 0; r < R; ++r) v[q + r * B] = w[r];  // position j + r N/R: natural order
    } else {
      // base and r NS occupy disjoint bits, and swz_mask is linear over GF(2):
      // swz(base + r NS) = (base + r NS) ^ swz_mask(base >> 4) ^ swz_mask(r NS >> 4)
      const uint32_t base = (j / NS) * NS * R + k;
      const uint32_t xb = swz_mask(base >> 4);
#pragma unroll
      for (int r = 0; r < R; ++r) line[(base + r * NS) ^ xb ^ swz_mask((uint32_t(r) * NS) >> 4)] = w[r];
    }
  }
  if (!LAST) {
    __syncwarp();
    const uint32_t lx = swz(lane);
#pragma unroll
    for (int i = 0; i < V; ++i) v[i] = line[V >= 16 ? swz_at(lx, i) : swz(lane + 32 * i)];
    __syncwarp();
  }
}

template <int V, int S, int NS>
__device__ __forceinline__ void warp_fft_from(float2 (&v)[V], float2 *line, const float2 *tw, uint32_t lane) {
  using P = WarpPlan<V>;
  if constexpr (S < P::NSTAGES) {
    constexpr int R = P::radix(S);
    warp_stage<V, R, NS, S + 1 == P::NSTAGES>(v, line, tw, lane);
    warp_fft_from<V, S + 1, NS * R>(v, line, tw, lane);
  }
}

template <int V>
__device__ __forceinline__ void warp_fft(float2 (&v)[V], float2 *line, const float2 *tw, uint32_t lane) {
  warp_fft_from<V, 0, 1>(v, line, tw, lane);
}

// Row pass (x axis): one warp per contiguous row, straight from and to HBM.
struct RowPassParams {
  float2 *data;
  uint32_t rows;       // rows in all volumes
  const float2 *tw;
  uint32_t rows_per_vol;
  size_t vstride;      // elements between volumes
};

template <int V>
__global__ void __launch_bounds__(256) k_fft_rows(RowPassParams p) {
  constexpr int N = 32 * V;
  extern __shared__ float2 smem[];
  float2 *tws = smem;                              // N
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2 *line = smem + N + warp * N;
  warp_twiddles<V>(tws, p.tw);
  __syncthreads();
  const uint32_t row = blockIdx.x * (blockDim.x >> 5) + warp;
  if (row >= p.rows) return;
  float2 *r = p.data + size_t(row / p.rows_per_vol) * p.vstride + size_t(row % p.rows_per_vol) * N;
  float2 v[V];
#pragma unroll
  for (int i = 0; i < V; ++i) v[i] = r[lane + 32 * i];
  warp_fft<V>(v, line, tws, lane);
#pragma unroll
  for (int i = 0; i < V; ++i) r[lane + 32 * i] = v[i];
}

// Column pass (y or z axis): a block owns TX = (warps) consecutive x columns
// of one (plane or row, volume); the tile [N][TX] is loaded with cp.async in
// rows of TX * 8 bytes into per-column padded lines, each warp transforms one
// column, and the tile is stored back in rows.
struct ColPassParams {
  float2 *data;
  uint32_t nx;         // columns per row
  uint32_t others;     // lines per volume / nx (y: planes, z: ny)
  size_t vstride;      // elements per volume
  size_t ostride;      // stride between successive "other" indices
  uint32_t estride;    // stride between successive elements of a column
  const float2 *tw;
};

// Blocks per SM the register budget is set for: 32 registers a thread up to
// 256-point lines, 64 for 512, 128 for 1024.
__host__ __device__ constexpr int cols_min_blocks(int v, int tx) { return (v <= 8 ? 2048 : v == 16 ? 1024 : 512) / (tx * 32); }

template <int V, int TX>
__global__ void __launch_bounds__(TX * 32, cols_min_blocks(V, TX)) k_fft_cols(ColPassParams p) {
  constexpr uint32_t N = 32 * V, L = line_stride(N, TX), NT = TX * 32;
  extern __shared__ float2 smem[];
  float2 *tws = smem, *tile = smem + N;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t nxt = (p.nx + TX - 1) / TX;
  const uint32_t xt = blockIdx.x % nxt, other = blockIdx.x / nxt, x0 = xt * TX;
  const uint32_t valid = min(uint32_t(TX), p.nx - x0);
  float2 *g = p.data + size_t(blockIdx.y) * p.vstride + size_t(other) * p.ostride + x0;
  const uint32_t l = threadIdx.x % TX, i0 = threadIdx.x / TX;  // compile-time TX: shifts
  constexpr uint32_t ISTEP = NT / TX;
  static_assert(ISTEP == 32 && N / ISTEP == V, "tile rows are i0 + 32 k");
  const uint32_t ix = swz(i0);
  const size_t s32 = size_t(32) * p.estride;
  float2 *gl = g + l + size_t(i0) * p.estride;
  float2 *tl = tile + l * L;
  // rows i0 + 32 (k0 + u), u < 4: swz_at(ix, k0 + u) = swz_at(ix, k0) ^ 32 u ^ swz_mask(2 u).
  // (Lines of up to 256 points measured faster with the plain swizzle, here
  // and in the warp FFT's exchanges.)
  if (l < valid) {
    if constexpr (V >= 16) {
      for (int k0 = 0; k0 < V; k0 += 4) {
        const uint32_t t0 = swz_at(ix, k0);
#pragma unroll
        for (int u = 0; u < 4; ++u) cp_async8(&tl[t0 ^ (32u * u) ^ swz_mask(2u * u)], gl + (k0 + u) * s32);
      }
    } else {
#pragma unroll 4
      for (uint32_t i = i0; i < N; i += ISTEP) cp_async8(&tile[l * L + swz(i)], &g[l + i * p.estride]);
    }
  } else {
#pragma unroll
    for (int k = 0; k < V; ++k) tl[swz_at(ix, k)] = make_float2(0.f, 0.f);
  }
  warp_twiddles<V>(tws, p.tw);
  cp_async_wait_all();
  __syncthreads();
  float2 *line = tile + warp * L;  // one warp per column
  const uint32_t lx = swz(lane);
  float2 v[V];
#pragma unroll
  for (int i = 0; i < V; ++i) v[i] = line[V >= 16 ? swz_at(lx, i) : swz(lane + 32 * i)];
  __syncwarp();
  warp_fft<V>(v, line, tws, lane);
#pragma unroll
  for (int i = 0; i < V; ++i) line[V >= 16 ? swz_at(lx, i) : swz(lane + 32 * i)] = v[i];
  __syncthreads();
  if (l < valid) {
    if constexpr (V >= 16) {
      for (int k0 = 0; k0 < V; k0 += 4) {
        const uint32_t t0 = swz_at(ix, k0);
#pragma unroll
        for (int u = 0; u < 4; ++u) gl[(k0 + u) * s32] = tl[t0 ^ (32u * u) ^ swz_mask(2u * u)];
      }
    } else {
#pragma unroll 4
      for (uint32_t i = i0; i < N; i += ISTEP) g[l + i * p.estride] = tile[l * L + swz(i)];
    }
  }
}

// ---------------------------------------------------------------------------
// Column passes over TMA tiles (y or z axis).  Persistent blocks walk tiles
// of adjacent columns x N lines of one (plane or row, volume),
// double-buffered: the tensor-memory accelerator loads tile k+1
// (cp.async.bulk.tensor, completion on an mbarrier) while tile k is
// transformed, and stores each finished tile back with a bulk tensor store.
// A 16-column tile lands with the 128-byte swizzle (16-byte chunk c of line r
// at chunk c ^ (r & 7)), so a warp reads its two columns 2w, 2w+1 as one
// 16-byte chunk per line, eight lines per quarter-warp on eight distinct
// chunks: no bank conflicts, and no load/store unit work for the tile copies
// at all.  Each warp transforms its columns with the warp FFT through its own
// exchange line.  Three forms:
//  * k_fft_cols_tma: 8 warps, thread 0 issues the copies between tiles
//    (256-point lines with nx a multiple of 16 but not of 32);
//  * k_fft_cols_tma_ws<V, H, NST>: H 16-column halves per tile, NST tile
//    stages, 8 H compute warps and a producer warp (512 points: H = 1, two
//    stages; 256 points: H = 2, three or two stages);
//  * k_fft_cols_tma64: 8-column tiles with the 64-byte swizzle for
//    1024-point lines, one column per warp.
// (One column per warp on 16-column tiles measured slower: its 8-byte reads
// put two lanes on each bank pair.)
// ---------------------------------------------------------------------------
constexpr int kTmaCols = 16;       // columns per tile (128 bytes per line)
constexpr int kTmaWarps = kTmaCols / 2;

struct ColTmaParams {
  uint32_t ntiles;   // tiles in all volumes
  uint32_t nxt;      // tiles across x (nx / 16)
  uint32_t others;   // y pass: planes per volume; z pass: rows (ny)
  uint32_t axis;     // 1: lines along y (tensor dim 1), 2: along z (dim 2)
  const float2 *tw;  // twiddles of length N
  unsigned *error;   // bit 1: a tile copy did not complete within the wait limit; bit 2: the drain
                     // after that timeout did not see the block's issued copies land either
  // self-test of the bounded waits (cyr_selftest_wait_limit); 0 in normal use:
  uint32_t poll_limit;  // polls per wait (0: kTmaWaitPolls)
  uint32_t extra_tx;    // bytes expected beyond the tile's, so its phase never completes
  // z pass of k_fft_cols_tma_ws only: the planes a later kernel reads, or null
  // (every plane stored).  Bit g of word w of 16-column group (row, x / 16) at
  // smask[(row (nx / 16) + x / 16) mwords + w] marks planes 8 (32 w + g) ..
  // + 7 of those columns, the same in every volume.  A tile with no bit set is
  // neither loaded nor stored; otherwise only the marked 8-plane boxes are
  // stored (through the 8-plane store map).
  const uint32_t *smask;
  uint32_t mwords;
};

// Dynamic shared memory of k_fft_cols_tma: two tiles, the warps' exchange lines,
// twiddles, two mbarriers, and slack to align the tiles to 1024 bytes.
__host__ __device__ constexpr size_t cols_tma_smem(uint32_t n) {
  return 2 * size_t(n) * kTmaCols * 8 + size_t(kTmaWarps) * n * 8 + size_t(n) * 8 + 32 + 1024;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// Completes `bytes` of the current phase's expected transaction count without a
// copy.  Only the wait-limit self-test needs it: its loads deliver extra_tx
// bytes fewer than the barrier expects, and after the timeout the producer
// completes those bytes itself, so that its drain wait ends exactly when the
// copies it really issued have landed.
__device__ __forceinline__ void mbar_complete_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.complete_tx.relaxed.cta.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// After a timeout: waits (bounded) for the last phase issued on a stage, so
// the block does not release shared memory under copies still landing; sets
// bit 2 of the error word if even that wait runs out.
__device__ __forceinline__ void mbar_drain(uint64_t *bar, uint32_t parity, uint32_t limit, uint32_t extra_tx,
                                           unsigned *error);
// Waits for the phase with the given parity; false if it did not complete within `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void mbar_drain(uint64_t *bar, uint32_t parity, uint32_t limit, uint32_t extra_tx,
                                           unsigned *error) {
  if (extra_tx) mbar_complete_tx(bar, extra_tx);
  if (!mbar_wait(bar, parity, limit)) atomicOr(error, 2u);
}
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_4d(const CUtensorMap *map, int c0, int c1, int c2, int c3, const void *src) {
  asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4}], [%5];\n" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

constexpr uint32_t kTmaWaitPolls = 1u << 22;  // each poll suspends up to a hardware time limit

// Block-synchronous form: thread 0 issues the copies between the tiles' compute phases.
template <int V>
__global__ void __launch_bounds__(kTmaWarps * 32, 1) k_fft_cols_tma(const __grid_constant__ CUtensorMap tmap,
                                                                      ColTmaParams p) {
  constexpr uint32_t N = 32 * V, TILE = N * kTmaCols;  // float2 per tile
  constexpr uint32_t BOX = N < 256 ? N : 256, NBOX = N / BOX;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  float2 *tiles = reinterpret_cast<float2 *>(base);  // [2][N][16], swizzled
  float2 *lines = tiles + 2 * TILE;                  // [warps][N]
  float2 *tws = lines + kTmaWarps * N;               // [N]
  uint64_t *mbar = reinterpret_cast<uint64_t *>(tws + N);
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  warp_twiddles<V>(tws, p.tw);
  __syncthreads();
  auto coords = [&](uint32_t t, uint32_t b, int (&c)[4]) {
    const uint32_t rest = t / p.nxt;
    c[0] = int((t % p.nxt) * kTmaCols);
    c[3] = int(rest / p.others);
    if (p.axis == 1) {
      c[1] = int(b * BOX), c[2] = int(rest % p.others);
    } else {
      c[1] = int(rest % p.others), c[2] = int(b * BOX);
    }
  };
  auto issue_load = [&](uint32_t t, int s) {
    mbar_expect_tx(&mbar[s], TILE * 8 + p.extra_tx);
#pragma unroll
    for (uint32_t b = 0; b < NBOX; ++b) {
      int c[4];
      coords(t, b, c);
      tma_load_4d(tiles + s * TILE + b * BOX * kTmaCols, &tmap, c[0], c[1], c[2], c[3], &mbar[s]);
    }
  };
  uint32_t t = blockIdx.x, k = 0;
  if (threadIdx.x == 0 && t < p.ntiles) issue_load(t, 0);
  float2 *line = lines + warp * N;
  for (; t < p.ntiles; t += gridDim.x, ++k) {
    const int s = int(k & 1u);
    if (threadIdx.x == 0 && t + gridDim.x < p.ntiles) {
      bulk_wait_read_all();  // the store from the other stage has read its tile
      issue_load(t + gridDim.x, s ^ 1);
    }
    const uint32_t limit = p.poll_limit ? p.poll_limit : kTmaWaitPolls;
    const bool ok = mbar_wait(&mbar[s], (k >> 1) & 1u, limit);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicOr(p.error, 1u);
        // let the copies in flight land (bounded) before the block releases its shared memory
        mbar_drain(&mbar[s], (k >> 1) & 1u, limit, p.extra_tx, p.error);
        if (t + gridDim.x < p.ntiles) mbar_drain(&mbar[s ^ 1], ((k + 1) >> 1) & 1u, limit, p.extra_tx, p.error);
      }
      break;
    }
    unsigned char *tb = reinterpret_cast<unsigned char *>(tiles + s * TILE);
    float2 a[V], c2[V];
#pragma unroll
    for (int i = 0; i < V; ++i) {
      const uint32_t r = lane + 32 * i;
      const float4 q = *reinterpret_cast<const float4 *>(tb + r * 128 + ((warp ^ (r & 7u)) << 4));
      a[i] = make_float2(q.x, q.y);
      c2[i] = make_float2(q.z, q.w);
    }
    warp_fft<V>(a, line, tws, lane);
    warp_fft<V>(c2, line, tws, lane);
#pragma unroll
    for (int i = 0; i < V; ++i) {
      const uint32_t r = lane + 32 * i;
      *reinterpret_cast<float4 *>(tb + r * 128 + ((warp ^ (r & 7u)) << 4)) =
          make_float4(a[i].x, a[i].y, c2[i].x, c2[i].y);
    }
    fence_proxy_async();  // the generic-proxy writes become visible to the bulk store
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
      for (uint32_t b = 0; b < NBOX; ++b) {
        int c[4];
        coords(t, b, c);
        tma_store_4d(&tmap, c[0], c[1], c[2], c[3], tiles + s * TILE + b * BOX * kTmaCols);
      }
      bulk_commit();
    }
  }
  if (threadIdx.x == 0) bulk_wait_all();
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

// Warp-specialised form: H halves of 16 columns per tile (each its own
// swizzled N x 128-byte region), NST tile stages, 8 H compute warps (two
// columns each) and a producer warp.  Per stage s: full[s] completes when a
// tile's copies have landed (transaction count), empty[s] when the compute
// warps are done with it.  The producer stores a finished tile as soon as
// empty[s] completes and reloads the stage once that store has read it; the
// compute warps never wait on the copies' shared-memory reads and never meet
// at a block barrier.  With NST = 3 the loads run two tiles ahead of the
// compute, which hides their latency when the stores are few (the masked z
// pass).  Twiddles take N - R0 entries (warp_twiddles), so three stages of
// 256-point, 32-column tiles fit the 227 KB a block may hold.
template <int V, int H, int NST>
__host__ __device__ constexpr size_t cols_tma_ws_smem() {
  return size_t(NST) * H * (32 * V) * kTmaCols * 8 + size_t(8 * H) * (32 * V) * 8 +
         size_t(32 * V - WarpPlan<V>::radix(0)) * 8 + 16 * NST + 1024;
}

template <int V, int H, int NST, bool MASK = false>
__global__ void __launch_bounds__((8 * H + 1) * 32, 1) k_fft_cols_tma_ws(const __grid_constant__ CUtensorMap tmap,
                                                                          const __grid_constant__ CUtensorMap smap,
                                                                          ColTmaParams p) {
  constexpr uint32_t N = 32 * V, HALF = N * kTmaCols, TILE = H * HALF;  // float2 per half / tile
  constexpr uint32_t BOX = N < 256 ? N : 256, NBOX = N / BOX, NW = 8 * H;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  float2 *tiles = reinterpret_cast<float2 *>(base);  // [NST][H][N][16], each half swizzled
  float2 *lines = tiles + NST * TILE;                // [compute warps][N]
  float2 *tws = lines + NW * N;                      // [N - R0]
  uint64_t *full = reinterpret_cast<uint64_t *>(tws + (N - WarpPlan<V>::radix(0))), *empty = full + NST;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int st = 0; st < NST; ++st) {
      mbar_init(&full[st], 1);
      mbar_init(&empty[st], NW);
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  warp_twiddles<V>(tws, p.tw);
  __syncthreads();
  // p.nxt counts tiles of H * 16 columns
  auto coords = [&](uint32_t t, uint32_t h, uint32_t b, int (&c)[4]) {
    const uint32_t rest = t / p.nxt;
    c[0] = int(((t % p.nxt) * H + h) * kTmaCols);
    c[3] = int(rest / p.others);
    if (p.axis == 1) {
      c[1] = int(b * BOX), c[2] = int(rest % p.others);
    } else {
      c[1] = int(rest % p.others), c[2] = int(b * BOX);
    }
  };
  auto region = [&](uint32_t s, uint32_t h, uint32_t b) { return tiles + s * TILE + h * HALF + b * BOX * kTmaCols; };
  // first mask word of half h of tile t (z pass with a store mask)
  auto mask_at = [&](uint32_t t, uint32_t h) {
    const uint32_t row = (t / p.nxt) % p.others;
    return p.smask + (size_t(row) * p.nxt * H + (t % p.nxt) * H + h) * p.mwords;
  };
  // The block's tiles are walked in batches of 32 candidates: lane l of a warp
  // reads the mask words of candidate c0 + l gridDim.x (MW words per half,
  // p.mwords == MW whenever a mask is set), and a ballot lists the tiles with
  // a marked plane.  A tile none of whose planes is read later is neither
  // loaded nor stored; the producer and the compute warps take the same
  // decision from the same words, so their stage and phase counts stay in
  // step.  One round of loads per 32 tiles keeps the mask reads off the
  // compute warps' per-tile path.
  // Without a mask (MASK false: p.smask is ignored) every tile is taken, in
  // the same order.  body(t, words) runs once per taken tile and returns false
  // to stop the walk.
  constexpr uint32_t MW = (V + 7) / 8;
  auto walk = [&](auto &&body) {
    if constexpr (!MASK) {
      uint32_t all[H][MW];
#pragma unroll
      for (uint32_t h = 0; h < H; ++h)
#pragma unroll
        for (uint32_t w = 0; w < MW; ++w) all[h][w] = ~0u;
      for (uint32_t t = blockIdx.x; t < p.ntiles; t += gridDim.x)
        if (!body(t, all)) return;
    } else {
      for (uint32_t c0 = blockIdx.x; c0 < p.ntiles; c0 += 32u * gridDim.x) {
        const uint32_t tl = c0 + lane * gridDim.x;
        uint32_t wl[H][MW], any = 0;
#pragma unroll
        for (uint32_t h = 0; h < H; ++h)
#pragma unroll
          for (uint32_t w = 0; w < MW; ++w) {
            wl[h][w] = tl < p.ntiles ? __ldg(&mask_at(tl, h)[w]) : 0u;
            any |= wl[h][w];
          }
        uint32_t todo = __ballot_sync(0xffffffffu, tl < p.ntiles && any != 0u);
        while (todo) {
          const int j = __ffs(int(todo)) - 1;
          todo &= todo - 1u;
          uint32_t wt[H][MW];
#pragma unroll
          for (uint32_t h = 0; h < H; ++h)
#pragma unroll
            for (uint32_t w = 0; w < MW; ++w) wt[h][w] = __shfl_sync(0xffffffffu, wl[h][w], j);
          if (!body(c0 + uint32_t(j) * gridDim.x, wt)) return;
        }
      }
    }
  };
  if (warp == NW) {  // producer: lane 0 issues the copies, the warp reads the mask words
    auto store = [&](uint32_t t, uint32_t s, const uint32_t (&wm)[H][MW]) {
      if constexpr (!MASK) {
#pragma unroll
        for (uint32_t h = 0; h < H; ++h)
#pragma unroll
          for (uint32_t b = 0; b < NBOX; ++b) {
            int c[4];
            coords(t, h, b, c);
            tma_store_4d(&tmap, c[0], c[1], c[2], c[3], region(s, h, b));
          }
      } else {
        // the marked 8-plane boxes only: box g starts 8 g lines (g KB, a
        // multiple of the swizzle's 1024-byte period) into the half
#pragma unroll
        for (uint32_t h = 0; h < H; ++h) {
          int c[4];
          coords(t, h, 0, c);
#pragma unroll
          for (uint32_t w = 0; w < MW; ++w) {
            uint32_t bits = wm[h][w];
            while (bits) {
              const uint32_t g = 32u * w + uint32_t(__ffs(int(bits)) - 1);
              bits &= bits - 1u;
              tma_store_4d(&smap, c[0], c[1], int(8 * g), c[3], region(s, h, 0) + g * 8 * kTmaCols);
            }
          }
        }
      }
      bulk_commit();
    };
    bool ok = true;
    uint32_t k = 0;  // tiles taken by this block so far; tile k sits in stage k % NST
    const uint32_t limit = p.poll_limit ? p.poll_limit : kTmaWaitPolls;
    int last[NST];               // last tile count loaded into each stage, -1: none
    uint32_t held[NST];          // the tile each stage holds
    uint32_t hwords[NST][H][MW]; // and its mask words
#pragma unroll
    for (int st = 0; st < NST; ++st) last[st] = -1, held[st] = 0;
    if (!MASK && lane != 0) return;  // without a mask lane 0 walks the tiles alone
    walk([&](uint32_t t, const uint32_t (&wt)[H][MW]) {
        if (lane == 0) {
          const uint32_t s = k % NST;
          if (k >= NST) {  // the tile taken NST before occupies stage s: store it, let the store read it, then reload
            ok = mbar_wait(&empty[s], (k / NST - 1) & 1u, limit);
            if (ok) {
              store(held[s], s, hwords[s]);
              bulk_wait_read_all();
            }
          }
          if (ok) {
            mbar_expect_tx(&full[s], TILE * 8 + p.extra_tx);
            last[s] = int(k);
            held[s] = t;
#pragma unroll
            for (uint32_t h = 0; h < H; ++h)
#pragma unroll
              for (uint32_t w = 0; w < MW; ++w) hwords[s][h][w] = wt[h][w];
#pragma unroll
            for (uint32_t h = 0; h < H; ++h)
#pragma unroll
              for (uint32_t b = 0; b < NBOX; ++b) {
                int c[4];
                coords(t, h, b, c);
                tma_load_4d(region(s, h, b), &tmap, c[0], c[1], c[2], c[3], &full[s]);
              }
          }
        }
        if (MASK) ok = __shfl_sync(0xffffffffu, ok, 0) != 0;
        ++k;
        return ok;
    });
    if (lane != 0) return;
    // the last (up to) NST tiles
    for (uint32_t kk = k >= NST ? k - NST : 0u; ok && kk < k; ++kk) {
      const uint32_t s = kk % NST;
      ok = mbar_wait(&empty[s], (kk / NST) & 1u, limit);
      if (ok) store(held[s], s, hwords[s]);
    }
    if (!ok) {
      atomicOr(p.error, 1u);
      // the block must not release its shared memory under copies still landing
      for (int st = 0; st < NST; ++st)
        if (last[st] >= 0) mbar_drain(&full[st], (uint32_t(last[st]) / NST) & 1u, limit, p.extra_tx, p.error);
    }
    bulk_wait_all();
    return;
  }
  // compute warps: warp w owns columns 2 (w % 8), 2 (w % 8) + 1 of half w / 8
  float2 *line = lines + warp * N;
  const uint32_t cw = warp & 7u, hw = warp >> 3;
  const uint32_t limit = p.poll_limit ? p.poll_limit : kTmaWaitPolls;
  uint32_t k = 0;
  walk([&](uint32_t, const uint32_t (&wt)[H][MW]) {
      // with a store mask only the lines of the stored 8-plane boxes are written back
      uint32_t keep[MW];
#pragma unroll
      for (uint32_t w = 0; w < MW; ++w) keep[w] = H == 1 || hw == 0 ? wt[0][w] : wt[H - 1][w];
      const uint32_t s = k % NST;
      // the warp leaves together (the walk's ballots and shuffles need every lane)
      if (!__all_sync(0xffffffffu, mbar_wait(&full[s], (k / NST) & 1u, limit))) {
        if (lane == 0) atomicOr(p.error, 1u);
        return false;
      }
      unsigned char *tb = reinterpret_cast<unsigned char *>(tiles + s * TILE + hw * HALF);
      float2 a[V], c2[V];
#pragma unroll
      for (int i = 0; i < V; ++i) {
        const uint32_t r = lane + 32 * i;
        const float4 q = *reinterpret_cast<const float4 *>(tb + r * 128 + ((cw ^ (r & 7u)) << 4));
        a[i] = make_float2(q.x, q.y);
        c2[i] = make_float2(q.z, q.w);
      }
      warp_fft<V>(a, line, tws, lane);
      warp_fft<V>(c2, line, tws, lane);
#pragma unroll
      for (int i = 0; i < V; ++i) {
        const uint32_t r = lane + 32 * i;
        if ((keep[i / 8] >> ((r >> 3) & 31u)) & 1u)
          *reinterpret_cast<float4 *>(tb + r * 128 + ((cw ^ (r & 7u)) << 4)) =
              make_float4(a[i].x, a[i].y, c2[i].x, c2[i].y);
      }
      fence_proxy_async();  // the generic-proxy writes become visible to the bulk store
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      ++k;
      return true;
  });
}

// 1024-point lines: two 16-column stages do not fit shared memory, so tiles are
// 8 columns (64-byte lines, 64-byte swizzle: chunk c of line r at
// c ^ ((r >> 1) & 3)), 8 compute warps of one column each and a producer warp,
// with the same two-stage protocol as k_fft_cols_tma_ws.
__host__ __device__ constexpr size_t cols_tma64_smem(uint32_t n) {
  return 2 * size_t(n) * 8 * 8 + size_t(8) * n * 8 + size_t(n) * 8 + 32 + 1024;
}

template <int V>
__global__ void __launch_bounds__(9 * 32, 1) k_fft_cols_tma64(const __grid_constant__ CUtensorMap tmap,
                                                              ColTmaParams p) {
  constexpr uint32_t N = 32 * V, TILE = N * 8;  // float2 per tile (8 columns)
  constexpr uint32_t BOX = 256, NBOX = N / BOX, NW = 8;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  float2 *tiles = reinterpret_cast<float2 *>(base);  // [2][N][8], swizzled
  float2 *lines = tiles + 2 * TILE;                  // [compute warps][N]
  float2 *tws = lines + NW * N;                      // [N]
  uint64_t *full = reinterpret_cast<uint64_t *>(tws + N), *empty = full + 2;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    mbar_init(&empty[0], NW);
    mbar_init(&empty[1], NW);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  warp_twiddles<V>(tws, p.tw);
  __syncthreads();
  // p.nxt counts tiles of 8 columns
  auto coords = [&](uint32_t t, uint32_t b, int (&c)[4]) {
    const uint32_t rest = t / p.nxt;
    c[0] = int((t % p.nxt) * 8);
    c[3] = int(rest / p.others);
    if (p.axis == 1) {
      c[1] = int(b * BOX), c[2] = int(rest % p.others);
    } else {
      c[1] = int(rest % p.others), c[2] = int(b * BOX);
    }
  };
  auto region = [&](int s, uint32_t b) { return tiles + s * TILE + b * BOX * 8; };
  const uint32_t limit = p.poll_limit ? p.poll_limit : kTmaWaitPolls;
  if (warp == NW) {  // producer
    if (lane != 0) return;
    auto store = [&](uint32_t t, int s) {
#pragma unroll
      for (uint32_t b = 0; b < NBOX; ++b) {
        int c[4];
        coords(t, b, c);
        tma_store_4d(&tmap, c[0], c[1], c[2], c[3], region(s, b));
      }
      bulk_commit();
    };
    bool ok = true;
    uint32_t k = 0;
    int last[2] = {-1, -1};
    for (uint32_t t = blockIdx.x; t < p.ntiles && ok; t += gridDim.x, ++k) {
      const int s = int(k & 1u);
      if (k >= 2) {
        ok = mbar_wait(&empty[s], ((k >> 1) - 1) & 1u, limit);
        if (!ok) break;
        store(t - 2 * gridDim.x, s);
        bulk_wait_read_all();
      }
      mbar_expect_tx(&full[s], TILE * 8 + p.extra_tx);
      last[s] = int(k);
#pragma unroll
      for (uint32_t b = 0; b < NBOX; ++b) {
        int c[4];
        coords(t, b, c);
        tma_load_4d(region(s, b), &tmap, c[0], c[1], c[2], c[3], &full[s]);
      }
    }
    const uint32_t ntile = p.ntiles > blockIdx.x ? (p.ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0u;
    for (uint32_t kk = ntile >= 2 ? ntile - 2 : 0u; ok && kk < ntile; ++kk) {
      const int s = int(kk & 1u);
      ok = mbar_wait(&empty[s], (kk >> 1) & 1u, limit);
      if (ok) store(blockIdx.x + kk * gridDim.x, s);
    }
    if (!ok) {
      atomicOr(p.error, 1u);
      for (int st = 0; st < 2; ++st)
        if (last[st] >= 0) mbar_drain(&full[st], (uint32_t(last[st]) >> 1) & 1u, limit, p.extra_tx, p.error);
    }
    bulk_wait_all();
    return;
  }
  // compute warps: warp w owns column w
  float2 *line = lines + warp * N;
  const uint32_t half = (warp & 1u) << 3, chunk = warp >> 1;
  uint32_t k = 0;
  for (uint32_t t = blockIdx.x; t < p.ntiles; t += gridDim.x, ++k) {
    const int s = int(k & 1u);
    if (!mbar_wait(&full[s], (k >> 1) & 1u, limit)) {
      if (lane == 0) atomicOr(p.error, 1u);
      return;
    }
    unsigned char *tb = reinterpret_cast<unsigned char *>(tiles + s * TILE);
    float2 a[V];
#pragma unroll
    for (int i = 0; i < V; ++i) {
      const uint32_t r = lane + 32 * i;
      a[i] = *reinterpret_cast<const float2 *>(tb + r * 64 + ((chunk ^ ((r >> 1) & 3u)) << 4) + half);
    }
    warp_fft<V>(a, line, tws, lane);
#pragma unroll
    for (int i = 0; i < V; ++i) {
      const uint32_t r = lane + 32 * i;
      *reinterpret_cast<float2 *>(tb + r * 64 + ((chunk ^ ((r >> 1) & 3u)) << 4) + half) = a[i];
    }
    fence_proxy_async();
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
}

// Per-thread register FFT for short strided lines (N = 8..64, powers of two):
// one thread owns one y or z line, and consecutive threads take consecutive
// x, so each of a warp's N loads and N stores is one contiguous 256-byte
// segment and no shared memory is involved.  Radix-2 decimation in
// frequency, fully unrolled (every index is a compile-time constant); the
// result is read out in bit-reversed order.
__host__ __device__ constexpr int bitrev(int k, int bits) {
  int r = 0;
  for (int b = 0; b < bits; ++b)
    if ((k >> b) & 1) r |= 1 << (bits - 1 - b);
  return r;
}

template <int N>
__device__ __forceinline__ void fft_reg(float2 (&a)[N], const float2 *__restrict__ tw) {
#pragma unroll
  for (int len = N; len >= 2; len >>= 1) {
    const int half = len >> 1, step = N / len;
#pragma unroll
    for (int start = 0; start < N; start += len)
#pragma unroll
      for (int j = 0; j < half; ++j) {
        const float2 u = a[start + j], v = a[start + j + half];
        a[start + j] = cadd(u, v);
        const float2 d = csub(u, v);
        a[start + j + half] = j == 0 ? d : cmul(d, __ldg(&tw[j * step]));
      }
  }
}

struct ThreadPassParams {
  float2 *data;
  uint32_t nx;       // lines per row of lines (x)
  uint32_t others;   // rows of lines: ny (z pass) or nz (y pass)
  size_t ostride;    // elements between rows of lines: nx (z pass) or nx * ny (y pass)
  size_t estride;    // elements between the points of a line: nx * ny (z) or nx (y)
  size_t vstride;    // elements between volumes (blockIdx.y)
  const float2 *tw;  // W_N^m, m < N
};

template <int N>
__global__ void __launch_bounds__(128) k_fft_thread(ThreadPassParams p) {
  constexpr int BITS = N == 8 ? 3 : N == 16 ? 4 : N == 32 ? 5 : 6;
  const size_t lines = size_t(p.nx) * p.others;
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= lines) return;
  const uint32_t x = uint32_t(t % p.nx);
  float2 *g = p.data + size_t(blockIdx.y) * p.vstride + (t / p.nx) * p.ostride + x;
  float2 a[N];
#pragma unroll
  for (int i = 0; i < N; ++i) a[i] = g[i * p.estride];
  fft_reg<N>(a, p.tw);
#pragma unroll
  for (int k = 0; k < N; ++k) g[k * p.estride] = a[bitrev(k, BITS)];
}

// Tensor build fused with the z-axis FFT, keeping only the z planes the Ewald
// projection can read.  A block owns TX consecutive x columns at one y, over
// all z: it computes the nvol entry volumes for those columns into shared
// memory, transforms them along z, and writes planes [zlo, zlo + kz) of the
// SHIFTED z axis (plane zlo + q holds unshifted bin igor(zlo + q)) as
// out[v][q][y][x].  The x and y FFTs then run on kz planes instead of nz, and
// the full 3D spectrum is never written.
struct BuildZParams {
  BuildParams b;      // morphology, constants, window, mean, mode
  FftAxis az;         // z-axis plan (n = nz)
  uint32_t tx;        // columns per block
  uint32_t stage;     // warp form: stage the morphology tile in shared memory
  uint32_t zlo, kz;   // kept shifted planes
  float2 *out;        // [nvol][kz][ny][nx]
};

__device__ __forceinline__ uint32_t igor(uint32_t j, uint32_t n);

template <int MORPH, bool CONV>
__global__ void __launch_bounds__(kFftThreads, 2) k_build_fft_z(BuildZParams p, const MaterialConsts *__restrict__ mcp) {
  if (MORPH == 0 && conv_selected(p.b) != CONV) return;
  extern __shared__ float2 smem[];
  __shared__ MaterialConsts mc;
  load_consts(mc, mcp);
  const BuildParams &b = p.b;
  const uint32_t nz = p.az.n, TX = p.tx, S = TX + 1, nvol = b.nvol;
  const uint32_t vsz = nz * S;
  float2 *bufa = smem, *bufb = smem + nvol * vsz, *tws = smem + 2 * nvol * vsz;
  const uint32_t nxt = (b.nx + TX - 1) / TX;
  const uint32_t xt = blockIdx.x % nxt, y = blockIdx.x / nxt, x0 = xt * TX;
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < TX * nz; t += blockDim.x) {
    const uint32_t l = t % TX, z = t / TX, x = x0 + l;
    float2 v[6];
    if (x < b.nx) {
      voxel_values<MORPH, CONV>(b, mc, (size_t(z) * b.ny + y) * b.nx + x, x, y, z, v);
    } else {
#pragma unroll
      for (int c = 0; c < 6; ++c) v[c] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int c = 0; c < 6; ++c)
      if (uint32_t(c) < nvol) bufa[c * vsz + z * S + l] = v[c];
  }
  stage_twiddles(tws, p.az.tw, nz);
  __syncthreads();
  const float2 *res = stockham(bufa, bufb, p.az, tws, TX, S, nvol);
  const size_t plane = size_t(b.nx) * b.ny;
  for (uint32_t t = threadIdx.x; t < nvol * p.kz * TX; t += blockDim.x) {
    const uint32_t l = t % TX, rest = t / TX;
    const uint32_t q = rest % p.kz, v = rest / p.kz;
    const uint32_t x = x0 + l;
    if (x >= b.nx) continue;
    const uint32_t u = igor(p.zlo + q, nz);
    p.out[(size_t(v) * p.kz + q) * plane + size_t(y) * b.nx + x] = res[(v * nz + u) * S + l];
  }
}

// Warp-FFT form of k_build_fft_z for nz = 32 V (128, 256, 512): the block
// builds the nvol x TX z-lines of its TX columns into padded shared lines,
// each warp transforms whole lines in registers (no block barrier inside the
// transform), and the kept planes are stored in rows of TX columns.
template <int MORPH, bool CONV, int V, int TX>
__global__ void __launch_bounds__(256) k_build_fft_z_warp(BuildZParams p, const MaterialConsts *__restrict__ mcp) {
  if (MORPH == 0 && conv_selected(p.b) != CONV) return;
  constexpr uint32_t NZ = 32 * V, L = line_stride(NZ, TX);
  extern __shared__ float2 smem[];
  __shared__ MaterialConsts mc;
  load_consts(mc, mcp);
  const BuildParams &b = p.b;
  const uint32_t nvol = b.nvol;
  float2 *tws = smem, *lines = smem + NZ;
  const uint32_t nxt = (b.nx + TX - 1) / TX;
  const uint32_t xt = blockIdx.x % nxt, y = blockIdx.x / nxt, x0 = xt * TX;
  warp_twiddles<V>(tws, p.az.tw);
  // With p.stage the block's morphology tile [m][z][TX] is copied into shared
  // memory with 16-byte cp.async first, so all of its loads are in flight at once.
  const uint32_t nl = nvol * TX * L;
  float4 *tile = reinterpret_cast<float4 *>(lines + nl + (nl & 1));
  const float4 *src = CONV ? b.conv : b.vox;
  const uint32_t l = threadIdx.x % TX, z0 = threadIdx.x / TX;
  constexpr uint32_t ZSTEP = 256 / TX;
  const uint32_t x = x0 + l;
  const bool xin = x < b.nx;
  const size_t plane = size_t(b.nx) * b.ny;
  const float4 *col = src + size_t(y) * b.nx + x;  // material 0, z = 0 of this column
  if (p.stage) {
    if (xin)
      for (uint32_t m = 0; m < b.nmat; ++m)
        for (uint32_t z = z0; z < NZ; z += ZSTEP) {
          const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(&tile[(m * NZ + z) * TX + l]));
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(col + m * b.nvox + z * plane)
                       : "memory");
        }
    cp_async_wait_all();
  }
  __syncthreads();
  for (uint32_t z = z0; z < NZ; z += ZSTEP) {
    float2 v[6];
    if (xin) {
      float2 nt[6];
      if (p.stage)
        nt_entries_at<MORPH, CONV>(b, mc, tile + z * TX + l, size_t(NZ) * TX, nt);
      else
        nt_entries_at<MORPH, CONV>(b, mc, col + z * plane, b.nvox, nt);
      values_from_nt(b, nt, x, y, z, v);
    } else {
#pragma unroll
      for (int c = 0; c < 6; ++c) v[c] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int c = 0; c < 6; ++c)
      if (uint32_t(c) < nvol) lines[(c * TX + l) * L + swz(z)] = v[c];
  }
  __syncthreads();
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (uint32_t li = warp; li < nvol * TX; li += nwarps) {
    float2 *line = lines + li * L;
    const uint32_t lx = swz(lane);
    float2 v[V];
#pragma unroll
    for (int i = 0; i < V; ++i) v[i] = line[swz_at(lx, i)];
    __syncwarp();
    warp_fft<V>(v, line, tws, lane);
#pragma unroll
    for (int i = 0; i < V; ++i) line[swz_at(lx, i)] = v[i];
    __syncwarp();
  }
  __syncthreads();
  if (!xin) return;
  float2 *out = p.out + size_t(y) * b.nx + x;
  for (uint32_t c = 0; c < nvol; ++c) {
    const float2 *ln = lines + (c * TX + l) * L;
    float2 *oc = out + size_t(c) * p.kz * plane;
    for (uint32_t q = z0; q < p.kz; q += ZSTEP) oc[q * plane] = ln[swz(igor(p.zlo + q, NZ))];
  }
}

// ---------------------------------------------------------------------------
// 3. DC replacement value per volume (src/cudaMain.cu:123-176): the mean of
// the periodic neighbours of index 0 in the unshifted spectrum.  The Ewald
// gather substitutes it wherever it reads index 0; the spectrum itself is
// left untouched.
// ---------------------------------------------------------------------------
// The spectra are stored as planes: plane pz of volume v starts at
// spec + v * vstride + pz * nx * ny.  p0, p1, pn are the planes holding the
// unshifted z bins 0, 1 and nz-1.
// Mean of the DC bin's neighbours (4 in 2D, else 6) of one volume whose z
// planes of unshifted bins 0, 1 and nz-1 are p0, p1 and pn.
__device__ __forceinline__ float2 dc_mean(const float2 *__restrict__ V, uint32_t nx, uint32_t ny, uint32_t nz,
                                          uint32_t p0, uint32_t p1, uint32_t pn) {
  const size_t P = size_t(nx) * ny;
  const float2 *Z0 = V + size_t(p0) * P;
  float2 s = make_float2(0.f, 0.f);
  s = cadd(s, Z0[1]);
  s = cadd(s, Z0[nx]);
  s = cadd(s, Z0[nx - 1]);
  s = cadd(s, Z0[size_t(ny - 1) * nx]);
  float cnt = 4.f;
  if (nz > 1) {
    s = cadd(s, V[size_t(p1) * P]);
    s = cadd(s, V[size_t(pn) * P]);
    cnt = 6.f;
  }
  return make_float2(s.x / cnt, s.y / cnt);
}

__global__ void k_dc(const float2 *__restrict__ spec, uint32_t nvol, size_t vstride, uint32_t nx, uint32_t ny,
                     uint32_t nz, uint32_t p0, uint32_t p1, uint32_t pn, float2 *__restrict__ dc) {
  const uint32_t v = threadIdx.x;
  if (v >= nvol) return;
  dc[v] = dc_mean(spec + size_t(v) * vstride, nx, ny, nz, p0, p1, pn);
}

// ---------------------------------------------------------------------------
// 4. Ewald projection for every E angle at once.
//
// Per detector pixel (X, Y): the reference's float geometry
// (include/uniaxial.h:891-931, with correctly rounded float operations),
// the spectrum gathered at the Ewald planes through the "Igor" shift
// j -> (N/2 - j) mod N as index arithmetic (:570-613), the intensity
// |(k^2 I - Q Q^T) p|^2 (include/cudaUtils.h:268-296) with
// p = sum_b coef[a][b] * P_b for angle a, and the linear interpolation
// between the two planes (:800-803).  Writes images[a][P].
// ---------------------------------------------------------------------------
struct EwaldParams {
  const float2 *spec;     // [nvol][planes][ny][nx]
  const float2 *dc;       // [nvol]
  uint32_t nx, ny, nz;
  size_t nvox;            // volume stride of spec (elements)
  uint32_t zshifted;      // 1: plane q holds shifted z = zlo + q (nplanes planes); 0: plane = unshifted z
  uint32_t zlo, nplanes;
  unsigned int *errors;   // incremented when a needed plane is not stored
  uint32_t nbasis;        // 1..3
  float4 *gram;           // when set: Gram maps [NQ][gplane] (gram_at) instead of per-angle images
  size_t gplane;          // float4 per Gram plane (gram_plane_size(ny, nx))
  uint32_t vol[3][3];     // vol[c][b]: volume holding component c of basis b
  uint32_t nangles;
  const float *coef;      // [nangles][nbasis]
  float start, dx, dy, dz;
  const float *qx, *qy, *qz;  // q-grid tables (include/uniaxial.h:645-650)
  float kmag;
  float kx, ky, kz;       // k * kVector (float)
  float kvx, kvy, kvz;    // kVector
  uint32_t interp;        // 0 nearest, 1 linear
  uint32_t twod;
  float *images;          // [nangles][P]
};

__device__ __forceinline__ uint32_t igor(uint32_t j, uint32_t n) {
  const uint32_t h = n / 2;
  return j <= h ? h - j : n + h - j;
}

// Scattered field of one polarization basis vector: t = d p - Q (Q . p).
__device__ __forceinline__ void scatter_t(const float Q[3], float d, float2 p0, float2 p1, float2 p2, float2 t[3]) {
  const float2 qp = make_float2(Q[0] * p0.x + Q[1] * p1.x + Q[2] * p2.x, Q[0] * p0.y + Q[1] * p1.y + Q[2] * p2.y);
  t[0] = make_float2(d * p0.x - Q[0] * qp.x, d * p0.y - Q[0] * qp.y);
  t[1] = make_float2(d * p1.x - Q[1] * qp.x, d * p1.y - Q[1] * qp.y);
  t[2] = make_float2(d * p2.x - Q[2] * qp.x, d * p2.y - Q[2] * qp.y);
}

// Re(a . conj b) of two complex 3-vectors.
__device__ __forceinline__ float redot3(const float2 a[3], const float2 b[3]) {
  return a[0].x * b[0].x + a[0].y * b[0].y + a[1].x * b[1].x + a[1].y * b[1].y + a[2].x * b[2].x + a[2].y * b[2].y;
}

// Gram form of the angle loop.  The polarization of E angle a is
// p(a) = sum_b E_b(a) P_b over NB basis vectors P_b, and t is linear in p, so
//   I(a) = |sum_b E_b t_b|^2 = sum_{b,b'} E_b E_b' G_bb',  G_bb' = Re(t_b . conj t_b'),
// and the plane interpolation (linear in I) applies to G.  G is accumulated
// once per pixel; each angle then costs NB (NB + 1) / 2 multiply-adds.
template <int NB>
__device__ __forceinline__ void gram_add(const float Q[3], float d, const float2 (&P)[3][NB], float w,
                                         float (&G)[NB * (NB + 1) / 2]) {
  float2 t[NB][3];
#pragma unroll
  for (int b = 0; b < NB; ++b) scatter_t(Q, d, P[0][b], P[1][b], P[2][b], t[b]);
  int q = 0;
#pragma unroll
  for (int b = 0; b < NB; ++b)
#pragma unroll
    for (int b2 = b; b2 < NB; ++b2) G[q++] += w * redot3(t[b], t[b2]);
}

template <int NB>
__device__ __forceinline__ float gram_intensity(const float (&G)[NB * (NB + 1) / 2], const float *__restrict__ cf) {
  float e[NB];
#pragma unroll
  for (int b = 0; b < NB; ++b) e[b] = __ldg(&cf[b]);
  float I = 0.f;
  int q = 0;
#pragma unroll
  for (int b = 0; b < NB; ++b)
#pragma unroll
    for (int b2 = b; b2 < NB; ++b2) I += (b == b2 ? 1.f : 2.f) * e[b] * e[b2] * G[q++];
  return I;
}

// Gram planes hold the pixels of the rotation's source image (x < W, y < H,
// row-major index y W + x) in 4 x 2 blocks, one 128-byte line per block: the
// rotated bilinear taps of an 8 x 4 warp tile touch about 8 lines per load,
// where row order touches about 14.
__host__ __device__ inline size_t gram_plane_size(int W, int H) { return size_t((H + 1) / 2) * ((W + 3) / 4) * 8; }
__device__ __forceinline__ uint32_t gram_at(int x, int y, int W) {
  return ((uint32_t(y) >> 1) * ((uint32_t(W) + 3) >> 2) + (uint32_t(x) >> 2)) * 8 + ((uint32_t(y) & 1) << 2) +
         (uint32_t(x) & 3);
}

// Gram maps: NB = 1 or 2 -> one float4 plane (G00 [G01 G11]), NB = 3 -> two
// (G00 G01 G02 G11 | G12 G22); a NaN pixel stores NaN in every component.
template <int NB>
struct GramLayout {
  static constexpr int NG = NB * (NB + 1) / 2;
  static constexpr int NQ = (NG + 3) / 4;
};

// gm: the pixel's float4 in plane 0; plane q at gm + q * plane.
template <int NB>
__device__ __forceinline__ void gram_store(float4 *gm, size_t plane, const float (&G)[NB * (NB + 1) / 2]) {
  constexpr int NG = GramLayout<NB>::NG, NQ = GramLayout<NB>::NQ;
  float v[4 * NQ];
#pragma unroll
  for (int q = 0; q < 4 * NQ; ++q) v[q] = q < NG ? G[q] : 0.f;
#pragma unroll
  for (int q = 0; q < NQ; ++q) gm[q * plane] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}

template <int NB>
__device__ __forceinline__ void gram_store_nan(float4 *gm, size_t plane) {
  const float n = __int_as_float(0x7fc00000);
#pragma unroll
  for (int q = 0; q < GramLayout<NB>::NQ; ++q) gm[q * plane] = make_float4(n, n, n, n);
}

__device__ __forceinline__ float intensity(float Q0, float Q1, float Q2, float d, float2 p0, float2 p1, float2 p2) {
  // t = d p - Q (Q . p)
  const float2 qp = make_float2(Q0 * p0.x + Q1 * p1.x + Q2 * p2.x, Q0 * p0.y + Q1 * p1.y + Q2 * p2.y);
  const float2 t0 = make_float2(d * p0.x - Q0 * qp.x, d * p0.y - Q0 * qp.y);
  const float2 t1 = make_float2(d * p1.x - Q1 * qp.x, d * p1.y - Q1 * qp.y);
  const float2 t2 = make_float2(d * p2.x - Q2 * qp.x, d * p2.y - Q2 * qp.y);
  return t0.x * t0.x + t0.y * t0.y + t1.x * t1.x + t1.y * t1.y + t2.x * t2.x + t2.y * t2.y;
}

// Where detector pixel (X, Y) meets the Ewald sphere: false for a NaN pixel,
// else the plane(s) to read (shifted z indices Z0 [, Z1 = Z0 + 1 with weight
// w1]).  Every operation is in float with correct rounding, in the
// reference's order (include/uniaxial.h:720-760), so NaN masks agree exactly.
struct EwaldGeom {
  float start, dx, dy, dz;
  float kmag, kx, ky, kz;
  uint32_t nx, ny, nz;
  uint32_t interp, twod;
};

__device__ __forceinline__ bool ewald_geometry(const EwaldGeom &g, uint32_t X, uint32_t Y, uint32_t &Z0, uint32_t &Z1,
                                               float &w1, int &nplanes) {
  const float posx = __fadd_rn(g.start, __fmul_rn(float(X), g.dx));
  const float posy = __fadd_rn(g.start, __fmul_rn(float(Y), g.dy));
  const float ax = __fadd_rn(g.kx, posx), ay = __fadd_rn(g.ky, posy);
  const float val = __fsub_rn(__fsub_rn(__fmul_rn(g.kmag, g.kmag), __fmul_rn(ax, ax)), __fmul_rn(ay, ay));
  Z0 = Z1 = 0;
  w1 = 0.f;  // weight of plane Z1
  nplanes = 1;
  if ((val < 0.f) || (X == g.nx - 1) || (Y == g.ny - 1)) return false;
  const float posz = __fadd_rn(-g.kz, __fsqrt_rn(val));
  if (g.interp == 0) {
    if (!g.twod) {
      const float r = roundf(__fdiv_rn(__fsub_rn(posz, g.start), g.dz));  // round(), uniaxial.h:749
      Z0 = r <= 0.f ? 0u : uint32_t(r);
    }
    if (Z0 > g.nz - 1) return false;
  } else if (!g.twod) {
    const float tz = __fdiv_rn(__fsub_rn(posz, g.start), g.dz);
    Z0 = tz <= 0.f ? 0u : uint32_t(tz);
    // Z > Nz-1 is the reference's NaN rule; Z == Nz-1 would read outside the volume
    if (Z0 >= g.nz - 1) return false;
    Z1 = Z0 + 1;
    nplanes = 2;
    const float base = __fadd_rn(g.start, __fmul_rn(float(Z0), g.dz));
    w1 = __fdiv_rn(__fsub_rn(posz, base), g.dz);
  }
  return true;
}

template <int NB>
__global__ void __launch_bounds__(256) k_ewald_angles(EwaldParams p) {
  const size_t npix = size_t(p.nx) * p.ny;
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  const uint32_t Y = uint32_t(t / p.nx), X = uint32_t(t % p.nx);
  const EwaldGeom g{p.start, p.dx, p.dy, p.dz, p.kmag, p.kx, p.ky, p.kz, p.nx, p.ny, p.nz, p.interp, p.twod};
  uint32_t zs[2];
  float w1;
  int nplanes;
  const bool isnan_px = !ewald_geometry(g, X, Y, zs[0], zs[1], w1, nplanes);
  const float nanv = __int_as_float(0x7fc00000);
  float *img = p.images + t;
  // the rotation's image: width ny, so pixel t is (x, y) = (t % ny, t / ny)
  float4 *gm = p.gram ? p.gram + gram_at(int(t % p.ny), int(t / p.ny), int(p.ny)) : nullptr;
  if (isnan_px) {
    if (gm) {
      gram_store_nan<NB>(gm, p.gplane);
      return;
    }
    for (uint32_t a = 0; a < p.nangles; ++a) img[size_t(a) * npix] = nanv;
    return;
  }
  // gather the basis spectra at the (one or two) planes and accumulate their Gram matrix
  const uint32_t ux = igor(X, p.nx), uy = igor(Y, p.ny);
  const float d = p.kmag * p.kmag;
  float G[NB * (NB + 1) / 2] = {};
  for (int pl = 0; pl < nplanes; ++pl) {
    const uint32_t uz = p.twod ? 0u : igor(zs[pl], p.nz);
    uint32_t pz = uz;
    if (p.zshifted) {
      pz = zs[pl] - p.zlo;
      if (zs[pl] < p.zlo || pz >= p.nplanes) {  // the host's plane range missed this pixel
        atomicAdd(p.errors, 1u);
        if (gm) {
          gram_store_nan<NB>(gm, p.gplane);
          return;
        }
        for (uint32_t a = 0; a < p.nangles; ++a) img[size_t(a) * npix] = nanv;
        return;
      }
    }
    const bool is_dc = ux == 0 && uy == 0 && uz == 0;
    const size_t idx = size_t(ux) + size_t(uy) * p.nx + size_t(pz) * p.nx * p.ny;
    float2 P[3][NB];
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const uint32_t v = p.vol[c][b];
        P[c][b] = is_dc ? p.dc[v] : __ldg(&p.spec[size_t(v) * p.nvox + idx]);
      }
    const float Q[3] = {p.kx + p.qx[X], p.ky + p.qy[Y], p.kz + (p.twod ? 0.f : p.qz[zs[pl]])};
    gram_add<NB>(Q, d, P, nplanes == 2 ? (pl == 0 ? 1.f - w1 : w1) : 1.f, G);
  }
  if (gm) {
    gram_store<NB>(gm, p.gplane, G);
    return;
  }
  for (uint32_t a = 0; a < p.nangles; ++a) img[size_t(a) * npix] = gram_intensity<NB>(G, p.coef + size_t(a) * NB);
}

// ---------------------------------------------------------------------------
// 5. Bilinear warp with the semantics of nppiWarpAffine_32f_C1R +
// NPPI_INTER_LINEAR (src/cudaMain.cu:858, :943): source = A dst in float as
// fma(a00, x, a01*y) + a02; written only if the source point lies in
// [0, W-1] x [0, H-1]; neighbours clamped; lerp in fma form.
// ---------------------------------------------------------------------------
struct WarpCoef {
  float a00, a01, a02, a10, a11, a12;
};

// Source corners and fractions of destination pixel (xd, yd); false when the
// source point lies outside the image (the destination keeps its value).
struct WarpTap {
  int x0, x1, y0, y1;  // corner columns and rows (row-major image, width W)
  float fx, fy;
};

__device__ __forceinline__ bool warp_tap(int W, int H, const WarpCoef &c, int xd, int yd, WarpTap &tp) {
  const float fx_ = float(xd), fy_ = float(yd);
  const float xs = __fadd_rn(__fmaf_rn(c.a00, fx_, __fmul_rn(c.a01, fy_)), c.a02);
  const float ys = __fadd_rn(__fmaf_rn(c.a10, fx_, __fmul_rn(c.a11, fy_)), c.a12);
  if (!(xs >= 0.f && xs <= float(W - 1) && ys >= 0.f && ys <= float(H - 1))) return false;
  const int x0 = min(int(floorf(xs)), W - 1), y0 = min(int(floorf(ys)), H - 1);
  const int x1 = min(x0 + 1, W - 1), y1 = min(y0 + 1, H - 1);
  tp.x0 = x0, tp.x1 = x1, tp.y0 = y0, tp.y1 = y1;
  tp.fx = __fsub_rn(xs, float(x0)), tp.fy = __fsub_rn(ys, float(y0));
  return true;
}

// NPP's bilinear blend of the four corners A (y0 x0), B (y0 x1), C (y1 x0), D (y1 x1).
__device__ __forceinline__ float warp_blend(float fx, float fy, float A, float B, float C, float D) {
  const float gx = __fsub_rn(1.f, fx), gy = __fsub_rn(1.f, fy);
  const float t0 = __fmaf_rn(gx, A, __fmul_rn(fx, B));
  const float t1 = __fmaf_rn(gx, C, __fmul_rn(fx, D));
  return __fmaf_rn(gy, t0, __fmul_rn(fy, t1));
}

__device__ __forceinline__ bool warp_sample(const float *__restrict__ src, int W, int H, const WarpCoef &c, int xd,
                                            int yd, float &out) {
  const float fx_ = float(xd), fy_ = float(yd);
  const float xs = __fadd_rn(__fmaf_rn(c.a00, fx_, __fmul_rn(c.a01, fy_)), c.a02);
  const float ys = __fadd_rn(__fmaf_rn(c.a10, fx_, __fmul_rn(c.a11, fy_)), c.a12);
  if (!(xs >= 0.f && xs <= float(W - 1) && ys >= 0.f && ys <= float(H - 1))) return false;
  const int x0 = min(int(floorf(xs)), W - 1), y0 = min(int(floorf(ys)), H - 1);
  const int x1 = min(x0 + 1, W - 1), y1 = min(y0 + 1, H - 1);
  const float fx = __fsub_rn(xs, float(x0)), fy = __fsub_rn(ys, float(y0));
  const float A = src[size_t(y0) * W + x0], B = src[size_t(y0) * W + x1];
  const float C = src[size_t(y1) * W + x0], D = src[size_t(y1) * W + x1];
  const float gx = __fsub_rn(1.f, fx), gy = __fsub_rn(1.f, fy);
  const float t0 = __fmaf_rn(gx, A, __fmul_rn(fx, B));
  const float t1 = __fmaf_rn(gx, C, __fmul_rn(fx, D));
  out = __fmaf_rn(gy, t0, __fmul_rn(fy, t1));
  return true;
}

// blockIdx.y selects image src + y * src_stride -> dst + y * dst_stride.
__global__ void k_warp(const float *__restrict__ src, float *__restrict__ dst, int W, int H, WarpCoef c,
                       size_t src_stride = 0, size_t dst_stride = 0) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= size_t(W) * H) return;
  src += blockIdx.y * src_stride;
  dst += blockIdx.y * dst_stride;
  float v;
  if (warp_sample(src, W, H, c, int(t % W), int(t / W), v)) dst[t] = v;
}

// Angle sums in float-float arithmetic: Knuth's TwoSum keeps hi + lo equal to
// the running sum of the FP32 samples to about 2^-48 relative, so the final
// float(sum / n) agrees with the reference's FP64 accumulation
// (src/cudaMain.cu:887-905) except where the exact mean lies within ~1e-13 of
// a rounding boundary.  The FP32 pipe does it; GB300's FP64 pipe is 1/64 rate.
struct AngleSum {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float s = __fadd_rn(hi, v);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(v, bp));
    hi = s;
    lo = __fadd_rn(lo, e);
  }
  __device__ __forceinline__ double value() const { return double(hi) + double(lo); }
};

// Mean over the angles as the reference forms it: with the rotation mask, NaN
// samples are skipped and counted out (0 when none is left); without it a
// NaN sample makes the mean NaN.
__device__ __forceinline__ float angle_mean(const AngleSum &s, uint32_t count, uint32_t nangles, uint32_t rot_mask) {
  if (rot_mask) return count == 0 ? 0.f : float(s.value() / double(count));
  return float(s.value() / double(nangles));
}

// Rotates every per-angle image, masks and sums over angles, and averages
// (src/cudaMain.cu:830-909, include/uniaxial.h:958-992).
struct RotateParams {
  const float *images;      // [batch = blockIdx.y][nangles][P]
  const WarpCoef *coef;     // [nangles]
  int W, H;                 // NPP image: width = Ny, height = Nx
  uint32_t nangles;
  uint32_t rot_mask;
  float *avg;               // [batch][P]
};

__global__ void __launch_bounds__(256) k_rotate_average(RotateParams p) {
  const size_t npix = size_t(p.W) * p.H;
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  const int xd = int(t % p.W), yd = int(t / p.W);
  const float *images = p.images + size_t(blockIdx.y) * p.nangles * npix;
  AngleSum sum;
  uint32_t count = 0;
  for (uint32_t a = 0; a < p.nangles; ++a) {
    float v = __int_as_float(0x7fc00000);
    warp_sample(images + size_t(a) * npix, p.W, p.H, p.coef[a], xd, yd, v);
    if (p.rot_mask) {
      if (isnan(v)) continue;
      ++count;
    }
    sum.add(v);
  }
  p.avg[size_t(blockIdx.y) * npix + t] = angle_mean(sum, count, p.nangles, p.rot_mask);
}

// Gram records: the Gram matrices of NEP energies of one pixel, energy s at
// float s * NG, padded to whole float4s and stored as RQ planes of float4
// ([group][RQ][plane], pixels placed by gram_at), so each of a warp's loads
// reads whole 16-byte pixels of one plane.  NEP = 1 is the per-energy layout (GramLayout); the
// field-spectrum path packs 12 floats per record (4 energies at NB = 2, 2 at
// NB = 3), so no load fetches padding.
template <int NB, int NEP>
struct GramRec {
  static constexpr int NG = NB * (NB + 1) / 2;
  static constexpr int RQ = (NEP * NG + 3) / 4;  // float4 per pixel
};

template <int NB>
__host__ __device__ constexpr int packed_energies() {
  return 12 / (NB * (NB + 1) / 2);
}

// Rotation and angle average from Gram maps (LAB frame): per angle a the
// corners' Gram matrices are blended as NPP blends intensities, then
// I(a) = sum_{b,b'} E_b(a) E_b'(a) G_bb' (the blend is linear, so this equals
// blending the per-angle intensities).  One thread forms one destination
// pixel for the NEP energies of its record group, so the tap arithmetic and
// each corner load serve all of them.  A NaN at any corner makes the blend
// NaN, so a tap with a corner outside its row's possibly-valid column range
// (the union over the group's energies of rows[e][y] = [x, y], conservative:
// every pixel outside is NaN) is a NaN sample without a load.
struct RotateGramParams {
  const float4 *gram;       // [group = blockIdx.y][RQ][plane] (gram_at)
  size_t plane;             // float4 per plane (gram_plane_size(W, H))
  const WarpCoef *coef;     // [nangles]
  const float *ecoef;       // [nangles][NB]
  const int2 *rows;         // [energy][H] from the launch's first energy, or null: no bound known
  int W, H;
  uint32_t nangles;
  uint32_t nenergies;       // energies of this launch (the last group may be partial)
  uint32_t rot_mask;
  float *avg;               // [energy][P]
};

// Blocks own 16 x 16 destination tiles (a warp: 8 x 4), so the rotated
// source taps of a warp stay within a few cache lines.
constexpr int kRotTile = 16;

template <int NB, int NEP>
__global__ void __launch_bounds__(kRotTile * kRotTile, 3) k_rotate_gram(RotateGramParams p) {
  constexpr int NG = GramRec<NB, NEP>::NG, RQ = GramRec<NB, NEP>::RQ;
  constexpr int U = RQ == 1 ? 4 : RQ == 2 ? 2 : 1;  // angles whose loads are issued together
  extern __shared__ int2 rows[];                    // [H] when p.rows is set
  const uint32_t group = blockIdx.y;
  const int ne = int(min(uint32_t(NEP), p.nenergies - group * NEP));
  if (p.rows)
    for (int y = int(threadIdx.x); y < p.H; y += int(blockDim.x)) {
      int2 r = p.rows[size_t(group) * NEP * p.H + y];
      for (int s = 1; s < ne; ++s) {
        const int2 q = p.rows[(size_t(group) * NEP + s) * p.H + y];
        r.x = min(r.x, q.x), r.y = max(r.y, q.y);
      }
      rows[y] = r;
    }
  __syncthreads();
  const size_t npix = size_t(p.W) * p.H;
  const int tiles_x = (p.W + kRotTile - 1) / kRotTile;
  const int warp = int(threadIdx.x >> 5), lane = int(threadIdx.x & 31);
  const int xd = int(blockIdx.x % tiles_x) * kRotTile + (warp & 1) * 8 + (lane & 7);
  const int yd = int(blockIdx.x / tiles_x) * kRotTile + (warp >> 1) * 4 + (lane >> 3);
  if (xd >= p.W || yd >= p.H) return;
  const float4 *gm = p.gram + size_t(group) * p.plane * RQ;
  AngleSum sum[NEP];
  uint32_t count[NEP];
#pragma unroll
  for (int s = 0; s < NEP; ++s) count[s] = 0;
  for (uint32_t a0 = 0; a0 < p.nangles; a0 += U) {
    WarpTap tp[U];
    bool in[U];
    float4 cv[U][4][RQ];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t a = a0 + u;
      in[u] = a < p.nangles && warp_tap(p.W, p.H, p.coef[a < p.nangles ? a : 0], xd, yd, tp[u]);
      if (in[u] && p.rows) {
        const int2 r0 = rows[tp[u].y0], r1 = rows[tp[u].y1];
        in[u] = tp[u].x0 >= r0.x && tp[u].x1 <= r0.y && tp[u].x0 >= r1.x && tp[u].x1 <= r1.y;
      }
      if (in[u]) {
        const uint32_t idx[4] = {gram_at(tp[u].x0, tp[u].y0, p.W), gram_at(tp[u].x1, tp[u].y0, p.W),
                                 gram_at(tp[u].x0, tp[u].y1, p.W), gram_at(tp[u].x1, tp[u].y1, p.W)};
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
          for (int q = 0; q < RQ; ++q) cv[u][c][q] = __ldg(&gm[q * p.plane + idx[c]]);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t a = a0 + u;
      if (a >= p.nangles) break;
      // per-angle weights of the Gram entries: E_b E_b' (x2 off the diagonal)
      float wq[NG];
      {
        float e[NB];
#pragma unroll
        for (int b = 0; b < NB; ++b) e[b] = __ldg(&p.ecoef[size_t(a) * NB + b]);
        int q = 0;
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
          for (int b2 = b; b2 < NB; ++b2) wq[q++] = (b == b2 ? 1.f : 2.f) * e[b] * e[b2];
      }
#pragma unroll
      for (int s = 0; s < NEP; ++s) {
        if (s >= ne) break;
        float v = __int_as_float(0x7fc00000);
        if (in[u]) {
          v = 0.f;
#pragma unroll
          for (int g = 0; g < NG; ++g) {
            const int f = s * NG + g, q = f / 4, r = f % 4;
            auto comp = [&](const float4 &x) { return r == 0 ? x.x : r == 1 ? x.y : r == 2 ? x.z : x.w; };
            const float G = warp_blend(tp[u].fx, tp[u].fy, comp(cv[u][0][q]), comp(cv[u][1][q]),
                                       comp(cv[u][2][q]), comp(cv[u][3][q]));
            v += wq[g] * G;
          }
        }
        if (p.rot_mask) {
          if (isnan(v)) continue;
          ++count[s];
        }
        sum[s].add(v);
      }
    }
  }
#pragma unroll
  for (int s = 0; s < NEP; ++s)
    if (s < ne) p.avg[(size_t(group) * NEP + s) * npix + size_t(yd) * p.W + xd] = angle_mean(sum[s], count[s], p.nangles, p.rot_mask);
}

// Detector warp of a request group's angle averages (one image per virtual
// energy ve = ve0 + blockIdx.y, request ve / e_per_req): the fill and the warp of
// k_fill + k_warp in one pass, written to that request's own projection.
__global__ void k_warp_group(const float *__restrict__ src, float *const *__restrict__ out_g, uint32_t e_per_req,
                             uint32_t ve0, int W, int H, WarpCoef c, float prefill) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const size_t npix = size_t(W) * H;
  if (t >= npix) return;
  const uint32_t ve = ve0 + blockIdx.y;  // src holds the launch's images from ve0 on
  float v;
  if (!warp_sample(src + size_t(blockIdx.y) * npix, W, H, c, int(t % W), int(t / W), v)) v = prefill;
  out_g[ve / e_per_req][size_t(ve % e_per_req) * npix + t] = v;
}

__global__ void k_fill(float *dst, size_t n, float v, size_t stride = 0) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t < n) dst[blockIdx.y * stride + t] = v;
}

}  // namespace cyr
