// Harness that runs the UNMODIFIED reference CUDA path (usnistgov/cyrsoxs
// v1.2.0.0, src/cudaMain.cu) on one case file and writes its raw output.
//
// Oracle infrastructure only: it produces the golden vectors that pin the CPU
// restatement in oracle/ and the GB300 kernels.  It is never linked into, or
// called by, the product.
//
// It drives the reference exactly the way its pybind11 front end does
// (src/pymain.cpp:47-67 computePolarizationDebug, :78-119 launch): the
// PYBIND-mode InputData setters (include/Input/InputData.h:430-615), the
// RefractiveIndexData::addData conversion n = 1 - delta + i*beta
// (include/PyClass/RefractiveIndex.h:101-106), then cudaMain / cudaMainStreams
// / computePolarization (include/cudaMain.h:53-87).
//
// Case file layout (little endian), written by tests/golden/cases.py:
//   char[8] "CYRCASE1"
//   u32 nx ny nz num_material num_energy num_k
//   u32 morphology_type windowing interpolation scatter_approach rot_mask
//       algorithm max_streams reference_frame(1 = LAB) case_type mode
//   f32 phys_size start_angle end_angle increment_angle pol_energy pol_eangle
//   f32 detector[3]
//   f32 energies[num_energy]          (ascending)
//   f32 kvecs[num_k*3]                (as given to setKVectors)
//   f32 optical[num_energy][num_material][4]  (delta_par beta_par delta_perp beta_perp)
//   f32 voxels[num_material][nz][ny][nx][4]    (the reference's Voxel::s1)
// Output: mode 0 -> f32/f64 projection [E][K][ny][nx];
//         mode 1 -> px, py, pz complex [nz][ny][nx] each, in Real precision.
//
// Timing (baseline measurement): `<case.bin> <out.bin> <repeats>` runs the
// mode-0 launch once untimed (CUDA context, cuFFT and NPP initialisation), then
// <repeats> more times, printing "seconds <t>" for each: the wall clock
// (std::chrono::steady_clock) around the whole cudaMain / cudaMainStreams call,
// which returns once the projections are in host memory.  The voxel and
// projection buffers are then pinned (cudaMallocHost), as the reference's
// command line allocates them (src/main.cpp:136, include/cudaHeaders.h:85).

#include <cudaMain.h>
#include <RotationMatrix.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

struct Reader {
  std::ifstream in;
  explicit Reader(const char *path) : in(path, std::ios::binary) {
    if (!in) throw std::runtime_error(std::string("cannot open ") + path);
  }
  template <class T>
  T get() {
    T v;
    in.read(reinterpret_cast<char *>(&v), sizeof(T));
    if (!in) throw std::runtime_error("truncated case file");
    return v;
  }
  std::vector<float> floats(size_t n) {
    std::vector<float> v(n);
    in.read(reinterpret_cast<char *>(v.data()), n * sizeof(float));
    if (!in) throw std::runtime_error("truncated case file");
    return v;
  }
};

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3 && argc != 4) {
    std::fprintf(stderr, "usage: %s <case.bin> <out.bin> [timed repeats]\n", argv[0]);
    return 2;
  }
  const int repeats = argc == 4 ? std::atoi(argv[3]) : 0;
  Reader r(argv[1]);
  char magic[8];
  r.in.read(magic, 8);
  if (std::memcmp(magic, "CYRCASE1", 8) != 0) {
    std::fprintf(stderr, "bad magic\n");
    return 2;
  }
  const uint32_t nx = r.get<uint32_t>(), ny = r.get<uint32_t>(), nz = r.get<uint32_t>();
  const uint32_t nmat = r.get<uint32_t>(), ne = r.get<uint32_t>(), nk = r.get<uint32_t>();
  const uint32_t morph = r.get<uint32_t>(), window = r.get<uint32_t>(), interp = r.get<uint32_t>();
  const uint32_t scatter = r.get<uint32_t>(), rotmask = r.get<uint32_t>(), algo = r.get<uint32_t>();
  const uint32_t streams = r.get<uint32_t>(), frame = r.get<uint32_t>(), casetype = r.get<uint32_t>();
  const uint32_t mode = r.get<uint32_t>();
  const float phys = r.get<float>(), a0 = r.get<float>(), a1 = r.get<float>(), da = r.get<float>();
  const float pol_energy = r.get<float>(), pol_eangle = r.get<float>();
  const std::vector<float> det = r.floats(3);
  const std::vector<float> energies = r.floats(ne);
  const std::vector<float> kvecs = r.floats(size_t(nk) * 3);
  const std::vector<float> optical = r.floats(size_t(ne) * nmat * 4);
  const size_t nvox = size_t(nx) * ny * nz;
  const std::vector<float> vox = r.floats(size_t(nmat) * nvox * 4);

  InputData in(static_cast<int>(nmat));
  in.setEnergies(std::vector<Real>(energies.begin(), energies.end()));
  in.setEAngles(a0, a1, da);
  in.setPhysSize(phys);
  in.setDimension({nx, ny, nz}, MorphologyOrder::XYZ);
  in.setCaseType(static_cast<CaseTypes>(casetype));
  if (casetype != CaseTypes::DEFAULT) {
    for (uint32_t i = 0; i < nk; ++i)
      in.setKVectors({kvecs[3 * i], kvecs[3 * i + 1], kvecs[3 * i + 2]});
  }
  if (casetype == CaseTypes::GRAZING_INCIDENCE) in.setDetectorCoordinates({det[0], det[1], det[2]});
  in.setMorphologyType(static_cast<MorphologyType>(morph));
  in.setAlgorithm(static_cast<int>(algo), static_cast<int>(streams));
  in.ewaldsInterpolation = static_cast<int>(interp);
  in.windowingType = window;
  in.rotMask = rotmask != 0;
  in.scatterApproach = scatter;
  in.referenceFrame = frame != 0;
  if (!in.validate()) {
    std::fprintf(stderr, "input data did not validate\n");
    return 3;
  }

  std::vector<Material> mats(size_t(ne) * nmat);
  for (size_t e = 0; e < ne; ++e)
    for (size_t m = 0; m < nmat; ++m) {
      const Real dpar = optical[(e * nmat + m) * 4 + 0], bpar = optical[(e * nmat + m) * 4 + 1];
      const Real dper = optical[(e * nmat + m) * 4 + 2], bper = optical[(e * nmat + m) * 4 + 3];
      mats[e * nmat + m].npara.x = 1 - dpar;
      mats[e * nmat + m].npara.y = bpar;
      mats[e * nmat + m].nperp.x = 1 - dper;
      mats[e * nmat + m].nperp.y = bper;
    }
  const size_t nvoxel_all = size_t(nmat) * nvox;
  Voxel *voxels = nullptr;
  std::vector<Voxel> voxels_pageable;
  if (repeats > 0) {
    if (cudaMallocHost(reinterpret_cast<void **>(&voxels), sizeof(Voxel) * nvoxel_all) != cudaSuccess) return 6;
  } else {
    voxels_pageable.resize(nvoxel_all);
    voxels = voxels_pageable.data();
  }
  for (size_t i = 0; i < nvoxel_all; ++i) {
    voxels[i].s1.x = vox[4 * i + 0];
    voxels[i].s1.y = vox[4 * i + 1];
    voxels[i].s1.z = vox[4 * i + 2];
    voxels[i].s1.w = vox[4 * i + 3];
  }

  RotationMatrix rm(&in);
  std::ofstream out(argv[2], std::ios::binary);
  if (mode == 0) {
    const size_t total = size_t(ne) * in.kVectors.size() * size_t(nx) * ny;
    std::vector<Real> proj_pageable;
    Real *proj = nullptr;
    if (repeats > 0) {
      if (cudaMallocHost(reinterpret_cast<void **>(&proj), sizeof(Real) * total) != cudaSuccess) return 6;
    } else {
      proj_pageable.assign(total, Real(0));
      proj = proj_pageable.data();
    }
    for (int call = 0; call <= repeats; ++call) {
      std::memset(proj, 0, sizeof(Real) * total);
      const auto t0 = std::chrono::steady_clock::now();
      int rc;
      if (in.algorithmType == Algorithm::CommunicationMinimizing)
        rc = cudaMain(in.voxelDims, in, mats, proj, rm, voxels);
      else
        rc = cudaMainStreams(in.voxelDims, in, mats, proj, rm, voxels);
      const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (rc != EXIT_SUCCESS) return 4;
      if (call > 0) std::printf("seconds %.6f\n", secs);
    }
    std::fflush(stdout);
    out.write(reinterpret_cast<const char *>(proj), total * sizeof(Real));
  } else {
    const auto &es = in.energies;
    const UINT eid = std::lower_bound(es.begin(), es.end(), Real(pol_energy)) - es.begin();
    std::vector<Complex> px(nvox), py(nvox), pz(nvox);
    const int rc = computePolarization(in.voxelDims, in, mats, px.data(), py.data(), pz.data(), rm,
                                       voxels, Real(pol_eangle), eid, static_cast<int>(nmat));
    if (rc != EXIT_SUCCESS) return 4;
    out.write(reinterpret_cast<const char *>(px.data()), nvox * sizeof(Complex));
    out.write(reinterpret_cast<const char *>(py.data()), nvox * sizeof(Complex));
    out.write(reinterpret_cast<const char *>(pz.data()), nvox * sizeof(Complex));
  }
  return out ? 0 : 5;
}
