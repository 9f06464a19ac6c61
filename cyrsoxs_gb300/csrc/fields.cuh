// Field-spectrum form of the scattering path: the morphology's energy
// independent fields are transformed once per request and every energy and
// E angle is formed from them at the Ewald sample points.
//
// Per material m the uniaxial tensor of a voxel is (include/uniaxial.h:82-151)
//   Nt_ij = A u_i^2 + B (|u|^2 - u_i^2) + C phi_ui      (i = j)
//   Nt_ij = D u_i u_j                                    (i != j)
// with u = sqrt(phi_a) s (phi_a s_i s_j = u_i u_j), so it is linear in the
// seven real fields u_x^2, u_y^2, u_z^2, u_x u_y, u_x u_z, u_y u_z, phi_ui,
// with energy dependent complex coefficients.  The FFT is linear, hence
//   FFT(Nt_v) = sum_g c_vg(E) FFT(F_g),
// exactly.  The diagonal coefficients share a common part R(E) (the base
// optical constants are the same for every material), which would cancel in
// the sum and amplify the FP32 rounding of the field spectra; it is taken out
// with one more field, T = sum_m (|u_m|^2 + phi_ui_m):
//   Nt_xx = sum_m [(D+B-R) u_x^2 + (B-R)(u_y^2 + u_z^2) + (C-R) phi_ui] + R T.
// The 7 M + 1 real fields are packed in pairs into complex volumes
// Z_j = F_2j + i F_2j+1 and transformed with the engine's complex 3D FFT; the
// Ewald kernel unpacks them with
//   F_2j(k) = (Z_j(k) + conj Z_j(-k)) / 2,  F_2j+1(k) = (Z_j(k) - conj Z_j(-k)) / 2i.
// Every field is windowed and has its volume mean removed before the FFT,
// which changes only bin 0; bin 0 is always replaced by the mean of its six
// (four in 2D) neighbours (src/cudaMain.cu:123-176), a symmetric stencil, so
// replacing it in each Z_j before unpacking is the same as replacing it in
// each tensor entry.
#pragma once

namespace cyr {

constexpr int kFieldsPerMaterial = 7;

__host__ __device__ constexpr uint32_t num_fields(uint32_t nmat) { return kFieldsPerMaterial * nmat + 1; }
__host__ __device__ constexpr uint32_t num_packed(uint32_t nmat) { return (num_fields(nmat) + 1) / 2; }

constexpr uint32_t kMaxFields = num_fields(kMaxMaterials);
constexpr uint32_t kMaxPacked = num_packed(kMaxMaterials);

// Field means from the per-material moments (k_moments over nsamp voxels), T
// last, computed by the calling block.  Any constant subtracted from a field
// changes only bin 0, which is replaced, so the means need only be close (a
// z-plane subsample suffices); they keep the FP32 rounding of the transform
// proportional to the fluctuations.
__device__ __forceinline__ void field_means(const double *__restrict__ mom, uint32_t nmat, size_t nsamp,
                                            float *__restrict__ out) {
  const uint32_t nf = num_fields(nmat);
  for (uint32_t g = threadIdx.x; g < nf; g += blockDim.x) {
    double v = 0.0;
    if (g + 1 < nf) {
      v = mom[(g / kFieldsPerMaterial) * kMoments + g % kFieldsPerMaterial];
    } else {
      for (uint32_t m = 0; m < nmat; ++m) {
        const double *M = mom + m * kMoments;
        v += M[0] + M[1] + M[2] + M[6];
      }
    }
    out[g] = float(v / double(nsamp));
  }
}

struct FieldParams {
  const float4 *vox;     // [nmat][nvox] as the reference stores Voxel::s1
  // request group (blockIdx.y = request): its morphologies, and the strides of
  // its moments and packed volumes; null for a single request
  const float4 *const *vox_g;
  size_t mom_stride, out_stride;
  uint32_t nx, ny, nz, nmat;
  size_t nvox;
  const double *mom;     // [nmat][kMoments] moment sums over nsamp voxels
  size_t nsamp;
  size_t i0, i1;         // voxels built: [i0, i1) (whole z planes)
  const float *hann_x, *hann_y, *hann_z;  // null when no windowing
  float2 *out;           // [num_packed][nvox]: field 2j in .x, field 2j+1 in .y
};

// Windowed, mean-free fields of every voxel, packed in pairs.
// Selects request blockIdx.y of a request group.
__device__ __forceinline__ void field_group(FieldParams &p) {
  if (!p.vox_g) return;
  p.vox = p.vox_g[blockIdx.y];
  p.mom += size_t(blockIdx.y) * p.mom_stride;
  p.out += size_t(blockIdx.y) * p.out_stride;
}

template <int MORPH>
__global__ void __launch_bounds__(256) k_build_fields(FieldParams p) {
  __shared__ float mean[kMaxFields];  // volume mean of each windowed field
  field_group(p);
  field_means(p.mom, p.nmat, p.nsamp, mean);
  __syncthreads();
  const size_t stride = size_t(gridDim.x) * blockDim.x;
  for (size_t i = p.i0 + size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < p.i1; i += stride) {
    float w = 1.f;
    if (p.hann_x) {
      const uint32_t x = uint32_t(i % p.nx), y = uint32_t((i / p.nx) % p.ny), z = uint32_t(i / (size_t(p.nx) * p.ny));
      w = p.hann_x[x] * p.hann_y[y] * p.hann_z[z];
    }
    float T = 0.f, pend = 0.f;
    uint32_t g = 0;
    float2 *o = p.out + i;
    // g is the same in every thread: the parity branches do not diverge
    auto emit = [&](float v) {
      v -= mean[g];
      if (g & 1u)
        o[size_t(g >> 1) * p.nvox] = make_float2(pend, v);
      else
        pend = v;
      ++g;
    };
    for (uint32_t m0 = 0; m0 < p.nmat; m0 += 4) {
      float4 sv[4];  // the loads of up to 4 materials are issued before any is used
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (m0 + u < p.nmat) sv[u] = __ldg(&p.vox[(m0 + u) * p.nvox + i]);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (m0 + u >= p.nmat) break;
        float sx, sy, sz, pa, pui;
        director<MORPH>(sv[u], sx, sy, sz, pa, pui);
        const float wa = w * pa;
        const float f0 = wa * sx * sx, f1 = wa * sy * sy, f2 = wa * sz * sz, f6 = w * pui;
        T += f0 + f1 + f2 + f6;
        emit(f0);
        emit(f1);
        emit(f2);
        emit(wa * sx * sy);
        emit(wa * sx * sz);
        emit(wa * sy * sz);
        emit(f6);
      }
    }
    emit(T);
    if (g & 1u) o[size_t(g >> 1) * p.nvox] = make_float2(pend, 0.f);
  }
}

// Field build fused with the x-row FFT (rows of N = 32 V points): a block owns
// one row (y, z) at a time and writes the row's packed fields into swizzled
// shared-memory lines, [npk][N] (the same fields, windowing and means as
// k_build_fields); each warp then loads a line into registers, runs the warp
// FFT with that line as its exchange buffer, and stores the transformed row.
// The packed volumes leave the chip once, already x-transformed: the build's
// write and the row pass's read-back of 8 npk bytes per voxel are gone.
// Shared memory: (npk + 1) N float2 (lines and twiddles).  Three blocks per SM
// (80 registers) measured faster than two blocks that also stage the next
// row's voxels in shared memory with cp.async.  (A hardware sine/cosine for
// the Euler angles saved 0.17 ms of 3.6 on the 256 x 512 x 512 request but
// doubled the full-size error against FP64, to 3.6e-5: not kept.)
__host__ __device__ constexpr size_t fields_rows_smem(uint32_t n, uint32_t npk, uint32_t nmat) {
  return (void)nmat, size_t(npk + 1) * n * sizeof(float2);
}

template <int MORPH, int V>
__global__ void __launch_bounds__(256, V <= 16 ? 3 : 1) k_build_fields_rows(FieldParams p, const float2 *__restrict__ tw_n,
                                                                            uint32_t npk) {
  constexpr uint32_t N = 32 * V;
  extern __shared__ float2 fsm[];
  float2 *tws = fsm;        // the warp FFT's stage twiddles (N - radix entries)
  float2 *lines = fsm + N;  // [npk][N]: element x of line j at lines[j N + swz(x)]
  __shared__ float mean[kMaxFields];
  field_group(p);
  field_means(p.mom, p.nmat, p.nsamp, mean);
  warp_twiddles<V>(tws, tw_n);
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const uint32_t nrows = uint32_t((p.i1 - p.i0) / N);
  for (uint32_t r = blockIdx.x; r < nrows; r += gridDim.x) {
    __syncthreads();  // means and twiddles ready; the previous row's lines consumed
    const size_t rowbase = p.i0 + size_t(r) * N;
    const uint32_t y = uint32_t((rowbase / N) % p.ny), z = uint32_t(rowbase / (size_t(N) * p.ny));
    const float wyz = p.hann_x ? p.hann_y[y] * p.hann_z[z] : 1.f;
    for (uint32_t x = threadIdx.x; x < N; x += blockDim.x) {
      const size_t i = rowbase + x;
      const float w = p.hann_x ? p.hann_x[x] * wyz : 1.f;
      float2 *o = lines + swz(x);
      float T = 0.f, pend = 0.f;
      uint32_t g = 0;
      auto emit = [&](float v) {
        v -= mean[g];
        if (g & 1u)
          o[(g >> 1) * N] = make_float2(pend, v);
        else
          pend = v;
        ++g;
      };
      for (uint32_t m0 = 0; m0 < p.nmat; m0 += 4) {
        float4 sv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (m0 + u < p.nmat) sv[u] = __ldg(&p.vox[(m0 + u) * p.nvox + i]);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (m0 + u >= p.nmat) break;
          float sx, sy, sz, pa, pui;
          director<MORPH>(sv[u], sx, sy, sz, pa, pui);
          const float wa = w * pa;
          const float f0 = wa * sx * sx, f1 = wa * sy * sy, f2 = wa * sz * sz, f6 = w * pui;
          T += f0 + f1 + f2 + f6;
          emit(f0);
          emit(f1);
          emit(f2);
          emit(wa * sx * sy);
          emit(wa * sx * sz);
          emit(wa * sy * sz);
          emit(f6);
        }
      }
      emit(T);
      if (g & 1u) o[(g >> 1) * N] = make_float2(pend, 0.f);
    }
    __syncthreads();
    for (uint32_t j = warp; j < npk; j += nw) {
      float2 *line = lines + j * N;
      float2 v[V];
      const uint32_t lx = swz(lane);
#pragma unroll
      for (int k = 0; k < V; ++k) v[k] = line[V >= 16 ? swz_at(lx, k) : swz(lane + 32 * k)];
      __syncwarp();
      warp_fft<V>(v, line, tws, lane);
      float2 *dst = p.out + size_t(j) * p.nvox + rowbase;
#pragma unroll
      for (int k = 0; k < V; ++k) dst[lane + 32 * k] = v[k];
    }
  }
}

// Ewald projection from the packed field spectra, for a batch of energies
// (blockIdx.y) and every E angle.  Per energy the unpacking and combination
// coefficients of tensor entry v (xx xy xz yy yz zz) and packed volume j are
// coef[e][v][j] = (alpha, beta):  Nt_v(k) = sum_j alpha Z_j(k) + beta conj Z_j(-k).
// Per angle a, the scattered polarization is p_c = sum_v M[a][c][v] Nt_v with
// a real 3 x 6 matrix (LAB frame: E_b on entry (c, b); MATERIAL frame: the
// rotation R^T folded in, include/uniaxial.h:163-165).
struct FieldEwaldParams {
  const float2 *zspec;   // [npk][nz][ny][nx], unshifted (natural) bin order
  const float2 *zdc;     // [npk] DC replacement of each packed volume (k_dc)
  uint32_t npk;
  size_t nvox;
  const float4 *coef;    // [ne][6][npk]: (alpha.x, alpha.y, beta.x, beta.y)
  const float *kmag;     // [ne]
  uint32_t e0;           // first energy of this batch
  float kvx, kvy, kvz;   // k vector
  EwaldGeom g;           // kmag, kx, ky, kz filled per energy
  const float *qx, *qy, *qz;
  uint32_t nangles;
  const float *mat;      // NB = 0: [nangles][3][6]
  const float *ecoef;    // NB > 0: [nangles][NB] E components of the LAB angle basis
  float *images;         // NB = 0: [batch][nangles][npix]
  float4 *gram;          // NB > 0: Gram records [batch / NEP][RQ][gplane] (GramRec<NB, packed_energies<NB>()>, gram_at)
  size_t gplane;         // float4 per Gram plane (gram_plane_size(ny, nx))
  uint32_t nbatch;       // energies of this launch
  // request group (k_ewald_fields<NB, true>): energy e belongs to request e / e_per_req, whose
  // packed volumes start at zspec + request * npk * nvox (DC at zdc + request * npk)
  uint32_t e_per_req;
};

// Structural zeros of the combination.  Tensor entry v (xx xy xz yy yz zz)
// takes field g = 7 m + f only when f is u_x^2, u_y^2, u_z^2 or phi_ui (the
// diagonal, which also takes T), u_x u_y (xy), u_x u_z (xz) or u_y u_z (yz)
// (include/uniaxial.h:94-151 in the contrast form above); coef[e][v][j] can
// be non-zero only when field 2j or 2j+1 enters entry v.  With 4 materials
// 34 of the 75 (entry, volume) pairs of the LAB frame's five entries are used.
__host__ __device__ constexpr bool field_enters(uint32_t nmat, int v, uint32_t g) {
  return g >= num_fields(nmat)        ? false                                    // T's zero partner
         : g + 1 == num_fields(nmat)  ? (v == 0 || v == 3 || v == 5)             // T
         : (v == 0 || v == 3 || v == 5) ? (g % kFieldsPerMaterial <= 2 || g % kFieldsPerMaterial == 6)
         : v == 1                     ? g % kFieldsPerMaterial == 3
         : v == 2                     ? g % kFieldsPerMaterial == 4
                                      : g % kFieldsPerMaterial == 5;             // v == 4
}
__host__ __device__ constexpr bool coef_used(uint32_t nmat, int v, uint32_t j) {
  return field_enters(nmat, v, 2 * j) || field_enters(nmat, v, 2 * j + 1);
}

constexpr int kEwaldEnergies = 4;  // energies (warps) per block
constexpr int kFieldEwaldThreads = 32 * kEwaldEnergies;
constexpr int kFieldGather = 4;  // packed volumes whose loads are issued together

// NB = 2 or 3: LAB frame, Gram maps over the E basis (p(a) = sum_b E_b(a) Nt e_b),
// rotated and averaged by k_rotate_gram.  NB = 0: any frame, p(a) = M(a) Nt per
// angle, per-angle images.  The energy is the fastest block index, so the
// blocks gathering one pixel tile for neighbouring energies (nearly the same
// Ewald sphere) run together and share the gathered sectors in L2.
// MT > 0: the morphology has MT materials and its coefficients keep the
// structural zeros (coef_used), so the volumes and entries are walked at
// compile time and the zero terms are never formed; MT = 0: any material
// count, every term formed.
template <int NB, bool GROUP = false, int MT = 0>
__global__ void __launch_bounds__(kFieldEwaldThreads) k_ewald_fields(FieldEwaldParams p) {
  // a block: 32 pixels x kEwaldEnergies neighbouring energies, one warp per
  // energy, so the warps of an SM gather nearly the same sectors (their Ewald
  // spheres almost coincide) and share them in L1
  extern __shared__ float4 fcoef_all[];  // [kEwaldEnergies][6][npk]
  const uint32_t ngrp = (p.nbatch + kEwaldEnergies - 1) / kEwaldEnergies;
  const uint32_t warp = threadIdx.x >> 5;
  const uint32_t eb = (blockIdx.x % ngrp) * kEwaldEnergies + warp, e = p.e0 + eb;
  const uint32_t nx = p.g.nx, ny = p.g.ny, nz = p.g.nz;
  for (uint32_t i = threadIdx.x; i < kEwaldEnergies * 6 * p.npk; i += blockDim.x) {
    const uint32_t w = i / (6 * p.npk), eg = (blockIdx.x % ngrp) * kEwaldEnergies + w;
    if (eg < p.nbatch) fcoef_all[i] = p.coef[size_t(p.e0 + eg) * 6 * p.npk + i % (6 * p.npk)];
  }
  __syncthreads();
  if (eb >= p.nbatch) return;
  constexpr uint32_t NPKC = MT > 0 ? num_packed(uint32_t(MT)) : 0u;
  const uint32_t npk = MT > 0 ? NPKC : p.npk;
  const float4 *fcoef = fcoef_all + warp * 6 * npk;
  const size_t npix = size_t(nx) * ny;
  const size_t t = size_t(blockIdx.x / ngrp) * 32 + (threadIdx.x & 31);
  if (t >= npix) return;
  const uint32_t Y = uint32_t(t / nx), X = uint32_t(t % nx);
  if (GROUP) {  // a request group (e_per_req > 0): this energy's request's packed volumes and DC
    const uint32_t rq = e / p.e_per_req;
    p.zspec += size_t(rq) * p.npk * p.nvox;
    p.zdc += size_t(rq) * p.npk;
  }
  EwaldGeom g = p.g;
  g.kmag = p.kmag[e];
  g.kx = __fmul_rn(g.kmag, p.kvx), g.ky = __fmul_rn(g.kmag, p.kvy), g.kz = __fmul_rn(g.kmag, p.kvz);
  uint32_t zs[2];
  float w1;
  int nplanes;
  float *img = p.images + size_t(eb) * p.nangles * npix + t;
  constexpr int NBG = NB > 0 ? NB : 1, NEP = packed_energies<NBG>();
  constexpr int NGG = GramRec<NBG, NEP>::NG, RQ = GramRec<NBG, NEP>::RQ;
  // component g of this energy: float f = (eb % NEP) NGG + g of the record, plane f / 4, lane f % 4
  // the rotation's image has width ny: pixel t is (x, y) = (t % ny, t / ny)
  float *gm = reinterpret_cast<float *>(p.gram + size_t(eb / NEP) * RQ * p.gplane +
                                        gram_at(int(t % ny), int(t / ny), int(ny)));
  const uint32_t f0 = (eb % NEP) * NGG;
  auto gput = [&](int g, float v) { gm[size_t((f0 + g) / 4) * p.gplane * 4 + (f0 + g) % 4] = v; };
  if (!ewald_geometry(g, X, Y, zs[0], zs[1], w1, nplanes)) {
    if constexpr (NB > 0) {
#pragma unroll
      for (int q = 0; q < NGG; ++q) gput(q, __int_as_float(0x7fc00000));
    } else {
      const float nanv = __int_as_float(0x7fc00000);
      for (uint32_t a = 0; a < p.nangles; ++a) img[size_t(a) * npix] = nanv;
    }
    return;
  }
  const uint32_t ux = igor(X, nx), uy = igor(Y, ny);
  const uint32_t mx = ux ? nx - ux : 0u, my = uy ? ny - uy : 0u;
  const float d = g.kmag * g.kmag;
  // Z_j(k) and Z_j(-k) at both planes: the loads of kFieldGather volumes of
  // both planes are issued together, and each coefficient serves both planes
  size_t i0[2], i1[2];
  bool is_dc[2];
#pragma unroll
  for (int pl = 0; pl < 2; ++pl) {
    const uint32_t uz = (g.twod || pl >= nplanes) ? 0u : igor(zs[pl], nz);
    const uint32_t mz = uz ? nz - uz : 0u;
    is_dc[pl] = ux == 0 && uy == 0 && uz == 0;
    i0[pl] = size_t(ux) + size_t(uy) * nx + size_t(uz) * npix;
    i1[pl] = size_t(mx) + size_t(my) * nx + size_t(mz) * npix;
  }
  const bool two = nplanes == 2;
  float2 N[2][6];
#pragma unroll
  for (int pl = 0; pl < 2; ++pl)
#pragma unroll
    for (int v = 0; v < 6; ++v) N[pl][v] = make_float2(0.f, 0.f);
  auto chunk = [&](uint32_t j0) {
    float2 za[2][kFieldGather], zb[2][kFieldGather];
#pragma unroll
    for (int q = 0; q < kFieldGather; ++q) {
      const uint32_t j = j0 + q;
#pragma unroll
      for (int pl = 0; pl < 2; ++pl) {
        za[pl][q] = zb[pl][q] = make_float2(0.f, 0.f);
        if (j < npk && (pl == 0 || two)) {
          if (is_dc[pl]) {
            za[pl][q] = zb[pl][q] = p.zdc[j];
          } else {
            const float2 *zj = p.zspec + size_t(j) * p.nvox;
            za[pl][q] = __ldg(&zj[i0[pl]]);
            zb[pl][q] = __ldg(&zj[i1[pl]]);
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < kFieldGather; ++q) {
      const uint32_t j = j0 + q;
      if (j >= npk) break;
#pragma unroll
      for (int v = 0; v < 6; ++v) {
        if (MT > 0 && !coef_used(uint32_t(MT), v, j)) continue;
        const float4 c = fcoef[v * npk + j];
#pragma unroll
        for (int pl = 0; pl < 2; ++pl) {
          const float2 a = za[pl][q], b = make_float2(zb[pl][q].x, -zb[pl][q].y);  // b = conj Z_j(-k)
          N[pl][v].x += c.x * a.x - c.y * a.y + c.z * b.x - c.w * b.y;
          N[pl][v].y += c.x * a.y + c.y * a.x + c.z * b.y + c.w * b.x;
        }
      }
    }
  };
  if constexpr (MT > 0) {
#pragma unroll
    for (uint32_t j0 = 0; j0 < NPKC; j0 += kFieldGather) chunk(j0);
  } else {
    for (uint32_t j0 = 0; j0 < npk; j0 += kFieldGather) chunk(j0);
  }
  float Q[2][3];
#pragma unroll
  for (int pl = 0; pl < 2; ++pl) {
    Q[pl][0] = g.kx + p.qx[X];
    Q[pl][1] = g.ky + p.qy[Y];
    Q[pl][2] = g.kz + ((g.twod || pl >= nplanes) ? 0.f : p.qz[zs[pl]]);
  }
  if constexpr (NB > 0) {
    constexpr int NG = NB * (NB + 1) / 2;
    float G[NG] = {};
    for (int pl = 0; pl < nplanes; ++pl) {
      // symmetric entry (c, b) of Nt: volumes xx xy xz yy yz zz
      float2 P[3][NB];
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        P[0][b] = N[pl][b == 0 ? 0 : b == 1 ? 1 : 2];
        P[1][b] = N[pl][b == 0 ? 1 : b == 1 ? 3 : 4];
        P[2][b] = N[pl][b == 0 ? 2 : b == 1 ? 4 : 5];
      }
      gram_add<NB>(Q[pl], d, P, two ? (pl == 0 ? 1.f - w1 : w1) : 1.f, G);
    }
#pragma unroll
    for (int q = 0; q < NG; ++q) gput(q, G[q]);
  } else {
    const float w0 = 1.f - w1;
    for (uint32_t a = 0; a < p.nangles; ++a) {
      const float *M = p.mat + size_t(a) * 18;
      float I[2];
      for (int pl = 0; pl < nplanes; ++pl) {
        float2 pc[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float2 acc = make_float2(0.f, 0.f);
#pragma unroll
          for (int v = 0; v < 6; ++v) acc = cfma(__ldg(&M[c * 6 + v]), N[pl][v], acc);
          pc[c] = acc;
        }
        I[pl] = intensity(Q[pl][0], Q[pl][1], Q[pl][2], d, pc[0], pc[1], pc[2]);
      }
      img[size_t(a) * npix] = two ? w0 * I[0] + w1 * I[1] : I[0];
    }
  }
}

// Planes of the packed field spectra that k_ewald_fields and k_dc read, as
// the store mask of the z pass (ColTmaParams::smask): per detector pixel, for
// every energy and k of the request, the planes ewald_geometry gives (the
// same float operations as k_ewald_fields, so the same planes) at the
// pixel's column and, for the unpacking's conj Z(-k), at the mirrored column
// and plane; plus the six neighbours of bin 0 that k_dc averages.  One bit per
// 8 planes and 16 columns; the words are zeroed by the caller.
constexpr uint32_t kZMaskMaxWords = 4;  // planes <= 1024
struct ZMaskParams {
  EwaldGeom g;          // kmag, kx, ky, kz set per energy and k
  const float *kmag;    // [ne]
  uint32_t ne;
  const float *kv;      // [nk][3] k vectors (float)
  uint32_t nk;
  uint32_t mwords;      // words per 16-column group
  uint32_t *mask;       // [ny][nx / 16][mwords]
};

__device__ __forceinline__ void zmask_set(const ZMaskParams &p, uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t g = z >> 3;
  atomicOr(&p.mask[(size_t(y) * (p.g.nx >> 4) + (x >> 4)) * p.mwords + (g >> 5)], 1u << (g & 31u));
}

__global__ void __launch_bounds__(256) k_zmask(ZMaskParams p) {
  const uint32_t nx = p.g.nx, ny = p.g.ny, nz = p.g.nz;
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t == 0) {  // the neighbours of bin 0 (dc_mean)
    zmask_set(p, 1 % nx, 0, 0);
    zmask_set(p, nx - 1, 0, 0);
    zmask_set(p, 0, 1 % ny, 0);
    zmask_set(p, 0, ny - 1, 0);
    zmask_set(p, 0, 0, 1 % nz);
    zmask_set(p, 0, 0, nz - 1);
  }
  if (t >= size_t(nx) * ny) return;
  const uint32_t Y = uint32_t(t / nx), X = uint32_t(t % nx);
  const uint32_t ux = igor(X, nx), uy = igor(Y, ny);
  const uint32_t mx = ux ? nx - ux : 0u, my = uy ? ny - uy : 0u;
  uint32_t own[kZMaskMaxWords] = {}, mir[kZMaskMaxWords] = {};
  for (uint32_t k = 0; k < p.nk; ++k) {
    const float kvx = p.kv[3 * k], kvy = p.kv[3 * k + 1], kvz = p.kv[3 * k + 2];
    for (uint32_t e = 0; e < p.ne; ++e) {
      EwaldGeom g = p.g;
      g.kmag = p.kmag[e];
      g.kx = __fmul_rn(g.kmag, kvx), g.ky = __fmul_rn(g.kmag, kvy), g.kz = __fmul_rn(g.kmag, kvz);
      uint32_t zs[2];
      float w1;
      int nplanes;
      if (!ewald_geometry(g, X, Y, zs[0], zs[1], w1, nplanes)) continue;
      for (int pl = 0; pl < nplanes; ++pl) {
        const uint32_t uz = igor(zs[pl], nz), mz = uz ? nz - uz : 0u;
        own[(uz >> 3) >> 5] |= 1u << ((uz >> 3) & 31u);
        mir[(mz >> 3) >> 5] |= 1u << ((mz >> 3) & 31u);
      }
    }
  }
  for (uint32_t w = 0; w < p.mwords && w < kZMaskMaxWords; ++w) {
    if (own[w]) atomicOr(&p.mask[(size_t(uy) * (nx >> 4) + (ux >> 4)) * p.mwords + w], own[w]);
    if (mir[w]) atomicOr(&p.mask[(size_t(my) * (nx >> 4) + (mx >> 4)) * p.mwords + w], mir[w]);
  }
}

}  // namespace cyr
