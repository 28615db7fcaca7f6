// Internal launchers shared by the C ABI translation units.
#pragma once

#include <string>

#include <cuda_runtime.h>

#include "bssn_fields.cuh"
#include "bssn_kernels.h"

struct BssnParams;

namespace bssn {

int fail(int code, const std::string& msg);
int cuda_status(cudaError_t e, const char* where);
int validate_params(const BssnParams* p);
int make_geo(const BssnParams* p, const int S[3], const int org[3], const int P[3], Geo& G);
Box box_of(const Geo& G);
Box full_box(const Geo& G);

cudaError_t launch_fill_periodic(double* u, int ncomp, const Geo& G, cudaStream_t s);
cudaError_t launch_fill_periodic(float* u, int ncomp, const Geo& G, cudaStream_t s);
cudaError_t launch_project(double* u, const Geo& G, const Box& B, cudaStream_t s);
cudaError_t launch_rk4_stage(const double* u0, const double* k, double* acc, double* out, const Geo& G,
                             const Box& B, int stage, double dt, int final_form, int project, cudaStream_t s);
cudaError_t launch_zero(double* u, long long n, cudaStream_t s);
cudaError_t rk4_step_patch(double* u0, double* ustage, double* k, double* acc, const RhsWork& w,
                           const Geo& G, const Box& B, bool fill, int final_form, cudaStream_t s,
                           const LowerTriangle* lower = nullptr);

}  // namespace bssn
