// The reference's C++ entry points over the GB300 engine's C ABI.
//
// usnistgov/cyrsoxs declares cudaMain, cudaMainStreams and computePolarization
// in include/cudaMain.h:53-87 and defines them in src/cudaMain.cu (cuFFT, NPP,
// cuBLAS).  A maintainer replaces src/cudaMain.cu with this file and links
// libcyrsoxs_gb300.so: src/main.cpp and src/pymain.cpp keep calling the same
// three functions, with the same arguments and the same EXIT_SUCCESS /
// EXIT_FAILURE results.  It compiles against the reference's own headers
// (include path of the reference tree) and this repository's include/.
//
// What crosses the boundary:
//  * InputData (include/Input/InputData.h:160-232) becomes cyr_options field
//    by field.  Energies are passed in InputData's order (the pybind setter
//    sorts them, InputData.h:443).
//  * Material holds n = 1 - delta + i beta (include/PyClass/RefractiveIndex.h:
//    101-106) per [energy][material]; the engine takes (delta, beta) back as
//    1 - Re n, exactly the value the reference's own n represents.
//  * Voxel::s1 (include/Input/Input.h:59-94) is already the engine's float4
//    layout [material][z][y][x].
//  * RotationMatrix is not read: the engine forms the k frames and E
//    rotations itself from InputData (the reference builds them from the same
//    fields, src/RotationMatrix.cpp:30-51).
//  * Errors: the reference exits the process (include/cudaHeaders.h:39-63); the
//    engine returns a status, which becomes EXIT_FAILURE with the message on
//    stderr.
//
// The FP64 build of the reference (-DDOUBLE_PRECISION, include/Datatypes.h:
// 33-46) maps onto the engine's double-precision entry points.

#include <cudaMain.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "cyrsoxs.h"

namespace {

struct Request {
  cyr_options opt{};
  std::vector<float> energies, kvecs;
#ifdef DOUBLE_PRECISION
  std::vector<double> optical;
#else
  std::vector<float> optical;
#endif
};

// InputData + materials -> options and optical constants [E][M][4] (delta_par, beta_par, delta_perp, beta_perp).
void make_request(const UINT *voxel, const InputData &in, const std::vector<Material> &mat, Request &r) {
  const size_t M = size_t(in.NUM_MATERIAL), E = in.energies.size();
  r.energies.assign(in.energies.begin(), in.energies.end());
  for (const Real3 &k : in.kVectors) {
    r.kvecs.push_back(float(k.x));
    r.kvecs.push_back(float(k.y));
    r.kvecs.push_back(float(k.z));
  }
  r.optical.resize(E * M * 4);
  for (size_t i = 0; i < E * M && i < mat.size(); ++i) {
    r.optical[4 * i + 0] = 1 - mat[i].npara.x;
    r.optical[4 * i + 1] = mat[i].npara.y;
    r.optical[4 * i + 2] = 1 - mat[i].nperp.x;
    r.optical[4 * i + 3] = mat[i].nperp.y;
  }
  cyr_options &o = r.opt;
  o.nx = voxel[0];
  o.ny = voxel[1];
  o.nz = voxel[2];
  o.num_material = uint32_t(M);
  o.num_energies = uint32_t(E);
  o.energies = r.energies.data();
  o.start_angle = float(in.startAngle);
  o.end_angle = float(in.endAngle);
  o.increment_angle = float(in.incrementAngle);
  o.phys_size = float(in.physSize);
  o.case_type = in.caseType;
  o.num_k = uint32_t(in.kVectors.size());
  o.k_vectors = r.kvecs.empty() ? nullptr : r.kvecs.data();
  o.detector[0] = float(in.detectorCoordinates.x);
  o.detector[1] = float(in.detectorCoordinates.y);
  o.detector[2] = float(in.detectorCoordinates.z);
  o.morphology_type = in.morphologyType;
  o.ewald_interpolation = uint32_t(in.ewaldsInterpolation);
  o.windowing = in.windowingType;
  o.scatter_approach = in.scatterApproach;
  o.algorithm = uint32_t(in.algorithmType);
  o.max_streams = uint32_t(in.numMaxStreams);
  o.rot_mask = in.rotMask ? 1u : 0u;
  o.reference_frame = in.referenceFrame ? 1u : 0u;
  o.strategy = CYR_STRATEGY_AUTO;
}

int status(int rc, const char *what) {
  if (rc == CYR_OK) return EXIT_SUCCESS;
  std::fprintf(stderr, "[cyrsoxs-gb300] %s failed: %s\n", what, cyr_last_error());
  return EXIT_FAILURE;
}

int run(const UINT *voxel, const InputData &in, const std::vector<Material> &mat, Real *projection,
        const Voxel *voxels, bool streams) {
  Request r;
  make_request(voxel, in, mat, r);
  const Real *vox = &voxels[0].s1.x;
#ifdef DOUBLE_PRECISION
  if (streams) r.opt.algorithm = 1;  // Algorithm 1: no windowing, as cyr_cuda_main_streams
  const int rc = cyr_cuda_main_fp64(&r.opt, r.optical.data(), vox, projection);
  return status(rc, streams ? "cudaMainStreams (FP64)" : "cudaMain (FP64)");
#else
  const int rc = streams ? cyr_cuda_main_streams(&r.opt, r.optical.data(), vox, projection)
                         : cyr_cuda_main(&r.opt, r.optical.data(), vox, projection);
  return status(rc, streams ? "cudaMainStreams" : "cudaMain");
#endif
}

}  // namespace

int cudaMain(const UINT *voxel, const InputData &idata, const std::vector<Material> &materialInput,
             Real *projectionAverage, RotationMatrix &, const Voxel *voxelInput) {
  return run(voxel, idata, materialInput, projectionAverage, voxelInput, false);
}

int cudaMainStreams(const UINT *voxel, const InputData &idata, const std::vector<Material> &materialInput,
                    Real *projectionAverage, RotationMatrix &, const Voxel *voxelInput) {
  return run(voxel, idata, materialInput, projectionAverage, voxelInput, true);
}

// EAngle is used as radians, as the reference's debug path does (src/cudaMain.cu:1716-1721).
int computePolarization(const UINT *voxel, const InputData &idata, const std::vector<Material> &materialInput,
                        Complex *polarizationX, Complex *polarizationY, Complex *polarizationZ, RotationMatrix &,
                        const Voxel *voxelInput, const Real EAngle, const UINT EnergyID, const int NUM_MATERIAL) {
  Request r;
  make_request(voxel, idata, materialInput, r);
  if (uint32_t(NUM_MATERIAL) != r.opt.num_material) {
    std::fprintf(stderr, "[cyrsoxs-gb300] computePolarization: NUM_MATERIAL %d differs from InputData's %u\n",
                 NUM_MATERIAL, r.opt.num_material);
    return EXIT_FAILURE;
  }
#ifdef DOUBLE_PRECISION
  const int rc = cyr_compute_polarization_fp64(&r.opt, r.optical.data(), &voxelInput[0].s1.x, EAngle, EnergyID,
                                               &polarizationX[0].x, &polarizationY[0].x, &polarizationZ[0].x);
#else
  const int rc = cyr_compute_polarization(&r.opt, r.optical.data(), &voxelInput[0].s1.x, EAngle, EnergyID,
                                          &polarizationX[0].x, &polarizationY[0].x, &polarizationZ[0].x);
#endif
  return status(rc, "computePolarization");
}

// warmup (include/cudaMain.h:97): the reference times a first CUDA call apart; the engine needs none.
int warmup() { return cyr_device_count() > 0 ? EXIT_SUCCESS : EXIT_FAILURE; }
