// cufft_rt.h -- the batched double-precision FFTs used beside the likelihood
// path (maximised likelihood, strain ingestion): cuFFT loaded at run time with
// dlopen, so that the engine builds and runs without it (the entry points that
// need it then return GWGPU_ECUDA with a message), and plans cached per
// context.
#pragma once

#include <cuda_runtime.h>

struct gwgpu_context;

namespace gwfft {

enum Type { kC2C = 0x29, kZ2Z = 0x69, kD2Z = 0x6a };  // cufftType values CUFFT_C2C, CUFFT_Z2Z, CUFFT_D2Z
constexpr int kForward = -1;             // CUFFT_FORWARD
constexpr int kInverse = 1;              // CUFFT_INVERSE (unnormalised)

// A plan of `batch` contiguous length-N transforms (input distance N, output
// distance N for Z2Z/C2C and N/2 + 1 for D2Z), reused across calls.  The cache
// holds at most 16 plans per context; creating one more destroys the others,
// so a caller fetches the plan it executes after any other plan it needs.
int plan(gwgpu_context *c, Type type, int N, int batch, int *out);
// Transforms on stream s (Z2Z / C2C in either direction, in place allowed; D2Z forward).
int exec_z2z(gwgpu_context *c, int plan, double2 *in, double2 *out, int direction, cudaStream_t s);
int exec_c2c(gwgpu_context *c, int plan, float2 *in, float2 *out, int direction, cudaStream_t s);
int exec_d2z(gwgpu_context *c, int plan, double *in, double2 *out, cudaStream_t s);
// Destroys the context's plans.
void release(gwgpu_context *c);

}  // namespace gwfft
