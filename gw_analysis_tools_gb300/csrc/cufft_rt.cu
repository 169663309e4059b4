// cufft_rt.cu -- run-time loaded cuFFT and the per-context plan cache.
#include "cufft_rt.h"

#include <dlfcn.h>

#include <map>
#include <mutex>
#include <tuple>

#include "capi_internal.h"

namespace gwfft {
namespace {

struct Lib {
  typedef int (*PlanMany)(int *, int, int *, int *, int, int, int *, int, int, int, int);
  typedef int (*ExecZ2Z)(int, void *, void *, int);
  typedef int (*ExecC2C)(int, void *, void *, int);
  typedef int (*ExecD2Z)(int, void *, void *);
  typedef int (*SetStream)(int, cudaStream_t);
  typedef int (*Destroy)(int);
  void *h = nullptr;
  PlanMany plan_many = nullptr;
  ExecZ2Z z2z = nullptr;
  ExecC2C c2c = nullptr;
  ExecD2Z d2z = nullptr;
  SetStream set_stream = nullptr;
  Destroy destroy = nullptr;
  bool ok = false;
};

Lib &lib() {
  static Lib f;
  static std::once_flag once;
  std::call_once(once, [] {
    const char *names[] = {"libcufft.so.12", "libcufft.so.13", "libcufft.so", "/usr/local/cuda/lib64/libcufft.so.12",
                           "/usr/local/cuda/lib64/libcufft.so"};
    for (const char *nm : names)
      if ((f.h = dlopen(nm, RTLD_NOW | RTLD_LOCAL))) break;
    if (!f.h) return;
    f.plan_many = (Lib::PlanMany)dlsym(f.h, "cufftPlanMany");
    f.z2z = (Lib::ExecZ2Z)dlsym(f.h, "cufftExecZ2Z");
    f.d2z = (Lib::ExecD2Z)dlsym(f.h, "cufftExecD2Z");
    f.c2c = (Lib::ExecC2C)dlsym(f.h, "cufftExecC2C");
    f.set_stream = (Lib::SetStream)dlsym(f.h, "cufftSetStream");
    f.destroy = (Lib::Destroy)dlsym(f.h, "cufftDestroy");
    f.ok = f.plan_many && f.z2z && f.d2z && f.c2c && f.set_stream && f.destroy;
  });
  return f;
}

constexpr size_t kMaxPlans = 16;  // per context
std::mutex g_mu;
std::map<gwgpu_context *, std::map<std::tuple<int, int, int>, int>> g_plans;

}  // namespace

int plan(gwgpu_context *c, Type type, int N, int batch, int *out) {
  Lib &f = lib();
  if (!f.ok) {
    c->last_error = "cuFFT library not found";
    return GWGPU_ECUDA;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  auto &m = g_plans[c];
  auto key = std::make_tuple((int)type, N, batch);
  auto it = m.find(key);
  if (it != m.end()) {
    *out = it->second;
    return GWGPU_OK;
  }
  if (m.size() >= kMaxPlans) {  // plans hold device work areas: bounded, oldest shapes dropped wholesale
    for (auto &kv : m) f.destroy(kv.second);
    m.clear();
  }
  int p = 0, n = N;
  const int odist = type == kD2Z ? N / 2 + 1 : N;
  if (f.plan_many(&p, 1, &n, nullptr, 1, N, nullptr, 1, odist, (int)type, batch) != 0) {
    c->last_error = "cuFFT plan";
    return GWGPU_ECUDA;
  }
  m[key] = p;
  *out = p;
  return GWGPU_OK;
}

int exec_z2z(gwgpu_context *c, int p, double2 *in, double2 *out, int direction, cudaStream_t s) {
  Lib &f = lib();
  if (f.set_stream(p, s) != 0 || f.z2z(p, in, out, direction) != 0) {
    c->last_error = "cuFFT exec";
    return GWGPU_ECUDA;
  }
  return GWGPU_OK;
}

int exec_c2c(gwgpu_context *c, int p, float2 *in, float2 *out, int direction, cudaStream_t s) {
  Lib &f = lib();
  if (f.set_stream(p, s) != 0 || f.c2c(p, in, out, direction) != 0) {
    c->last_error = "cuFFT exec";
    return GWGPU_ECUDA;
  }
  return GWGPU_OK;
}

int exec_d2z(gwgpu_context *c, int p, double *in, double2 *out, cudaStream_t s) {
  Lib &f = lib();
  if (f.set_stream(p, s) != 0 || f.d2z(p, in, out) != 0) {
    c->last_error = "cuFFT exec";
    return GWGPU_ECUDA;
  }
  return GWGPU_OK;
}

void release(gwgpu_context *c) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_plans.find(c);
  if (it == g_plans.end()) return;
  Lib &f = lib();
  if (f.ok)
    for (auto &kv : it->second) f.destroy(kv.second);
  g_plans.erase(it);
}

}  // namespace gwfft
