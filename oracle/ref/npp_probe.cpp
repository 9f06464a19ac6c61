// Black-box probe of nppiWarpAffine_32f_C1R_Ctx with NPPI_INTER_LINEAR, the
// library call the reference uses to rotate every Ewald projection
// (src/cudaMain.cu:848-875) and to apply the detector warp (:916-960).
//
// NPP is closed; its pixel-centre convention, edge rule and interpolation
// arithmetic are pinned here by running it on seeded images and storing the
// outputs as golden files (tests/golden/npp_warp_*.bin).  The oracle's and the
// GB300 kernel's warps are then checked against those files.  Oracle
// infrastructure only.
//
// Probe file layout (little endian), written by tests/golden/npp_cases.py:
//   char[8] "NPPPROBE"; u32 count;
//   per probe: u32 width, height; f64 coeffs[2][3]; f32 prefill; f32 src[height][width]
// Output: per probe f32 dst[height][width] (prefilled, then warped).

#include <cuda_runtime.h>
#include <npp.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <vector>

static NppStreamContext make_ctx() {
  NppStreamContext ctx{};
  cudaGetDevice(&ctx.nCudaDeviceId);
  cudaDeviceProp p;
  cudaGetDeviceProperties(&p, ctx.nCudaDeviceId);
  cudaDeviceGetAttribute(&ctx.nCudaDevAttrComputeCapabilityMajor, cudaDevAttrComputeCapabilityMajor,
                         ctx.nCudaDeviceId);
  cudaDeviceGetAttribute(&ctx.nCudaDevAttrComputeCapabilityMinor, cudaDevAttrComputeCapabilityMinor,
                         ctx.nCudaDeviceId);
  ctx.hStream = 0;
  ctx.nMultiProcessorCount = p.multiProcessorCount;
  ctx.nMaxThreadsPerMultiProcessor = p.maxThreadsPerMultiProcessor;
  ctx.nMaxThreadsPerBlock = p.maxThreadsPerBlock;
  ctx.nSharedMemPerBlock = p.sharedMemPerBlock;
  ctx.nStreamFlags = cudaStreamDefault;
  return ctx;
}

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s <probe.bin> <out.bin>\n", argv[0]);
    return 2;
  }
  std::ifstream in(argv[1], std::ios::binary);
  char magic[8];
  in.read(magic, 8);
  if (!in || std::memcmp(magic, "NPPPROBE", 8) != 0) {
    std::fprintf(stderr, "bad probe file\n");
    return 2;
  }
  uint32_t count = 0;
  in.read(reinterpret_cast<char *>(&count), 4);
  const NppStreamContext ctx = make_ctx();
  std::ofstream out(argv[2], std::ios::binary);
  for (uint32_t c = 0; c < count; ++c) {
    uint32_t w = 0, h = 0;
    double coeffs[2][3];
    float prefill = 0.f;
    in.read(reinterpret_cast<char *>(&w), 4);
    in.read(reinterpret_cast<char *>(&h), 4);
    in.read(reinterpret_cast<char *>(coeffs), sizeof(coeffs));
    in.read(reinterpret_cast<char *>(&prefill), 4);
    std::vector<float> src(size_t(w) * h), dst(size_t(w) * h, prefill);
    in.read(reinterpret_cast<char *>(src.data()), src.size() * 4);
    if (!in) {
      std::fprintf(stderr, "truncated probe %u\n", c);
      return 2;
    }
    float *d_src = nullptr, *d_dst = nullptr;
    if (cudaMalloc(&d_src, src.size() * 4) != cudaSuccess || cudaMalloc(&d_dst, dst.size() * 4) != cudaSuccess) {
      std::fprintf(stderr, "cudaMalloc failed\n");
      return 3;
    }
    cudaMemcpy(d_src, src.data(), src.size() * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_dst, dst.data(), dst.size() * 4, cudaMemcpyHostToDevice);
    const NppiSize size{static_cast<int>(w), static_cast<int>(h)};
    const NppiRect rect{0, 0, static_cast<int>(w), static_cast<int>(h)};
    const NppStatus st = nppiWarpAffine_32f_C1R_Ctx(d_src, size, static_cast<int>(w * 4), rect, d_dst,
                                                    static_cast<int>(w * 4), rect, coeffs, NPPI_INTER_LINEAR, ctx);
    cudaDeviceSynchronize();
    if (st < 0) {
      std::fprintf(stderr, "probe %u: NPP status %d\n", c, static_cast<int>(st));
      return 4;
    }
    cudaMemcpy(dst.data(), d_dst, dst.size() * 4, cudaMemcpyDeviceToHost);
    cudaFree(d_src);
    cudaFree(d_dst);
    out.write(reinterpret_cast<const char *>(dst.data()), dst.size() * 4);
  }
  return out ? 0 : 5;
}
