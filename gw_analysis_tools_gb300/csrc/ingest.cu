// ingest.cu -- the on-disk formats that feed the registered detector streams:
//
//  * GWOSC ("LOSC") strain text files and PSD tables (read_LOSC_data_file,
//    read_LOSC_PSD_file, count_lines_*; io_util.cpp:403-500, 682-714), parsed
//    natively: the whole file is read at once and its data lines are parsed in
//    parallel chunks;
//  * allocate_LOSC_data (io_util.cpp:523-664): trim to the PSD's observation
//    time around the trigger, Tukey window (util.cpp:1736-1757), forward DFT
//    times dt, keep the PSD's frequency band.  The window, the transform (one
//    batched cuFFT real-to-complex plan over the detectors) and the band
//    selection run on the device;
//  * populate_noise (detector_util.cpp:86-283) for the ground-detector curves:
//    the analytic aLIGO and Hanford O1 fits, and linear interpolation of the
//    tabulated curves (gsl_interp_linear) read from the caller's noise
//    directory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gwgpu.h"
#include "capi_internal.h"
#include "cufft_rt.h"

namespace {

// ------------------------------------------------------------- text parsing
bool read_whole(const char *path, std::string &out) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (n < 0) {
    std::fclose(f);
    return false;
  }
  out.resize((size_t)n + 1);
  size_t got = n ? std::fread(&out[0], 1, (size_t)n, f) : 0;
  std::fclose(f);
  out.resize(got);
  return got == (size_t)n;
}

// Lines as std::getline yields them: split at '\n'; a final newline does not
// start another line.
template <class F>
void for_lines(const char *b, const char *e, F &&fn) {
  while (b < e) {
    const char *nl = (const char *)std::memchr(b, '\n', (size_t)(e - b));
    const char *le = nl ? nl : e;
    fn(b, le);
    b = nl ? nl + 1 : e;
  }
}

long long count_lines(const std::string &s) {
  long long n = 0;
  for_lines(s.data(), s.data() + s.size(), [&](const char *, const char *) { n++; });
  return n;
}

// std::stod of the text [b, e): leading white space skipped, the longest
// number prefix converted, the rest ignored; false where stod would throw (no
// number, or out of range).
bool parse_double(const char *b, const char *e, double *v) {
  while (b < e && std::isspace((unsigned char)*b)) b++;
  if (b >= e) return false;
  const char *p = b;
  bool neg = false;
  if (*p == '+' || *p == '-') {
    neg = *p == '-';
    p++;
  }
  const bool hex = e - p >= 2 && p[0] == '0' && (p[1] == 'x' || p[1] == 'X');
  if (!hex && p < e && *p != '+' && *p != '-') {
    double x;
    auto r = std::from_chars(p, e, x, std::chars_format::general);
    if (r.ec == std::errc() && r.ptr != p) {
      *v = neg ? -x : x;
      return true;
    }
    if (r.ec == std::errc::result_out_of_range) return false;
  }
  // rare forms (hexadecimal, words from_chars does not take): the C library
  std::string tmp(b, e);
  char *endp = nullptr;
  errno = 0;
  double x = std::strtod(tmp.c_str(), &endp);
  if (endp == tmp.c_str() || errno == ERANGE) return false;
  *v = x;
  return true;
}

// Comma-separated items of one line as getline(lineStream, item, ',') yields
// them (an empty last item is not produced), each converted like stod.
bool parse_csv_line(const char *b, const char *e, std::vector<double> &out) {
  while (b < e) {
    const char *c = (const char *)std::memchr(b, ',', (size_t)(e - b));
    const char *ie = c ? c : e;
    double v;
    if (!parse_double(b, ie, &v)) return false;
    out.push_back(v);
    if (!c) break;
    b = c + 1;
  }
  return true;
}

// Every comma-separated value of the lines in [b, e), in order, parsed in
// parallel chunks split at line boundaries.
int parse_csv_block(const char *b, const char *e, std::vector<double> &out) {
  const size_t bytes = (size_t)(e - b);
  unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  int T = (int)std::min<size_t>(std::min<unsigned>(hw, 32u), bytes / (1u << 20) + 1);
  std::vector<const char *> cut(T + 1);
  cut[0] = b;
  cut[T] = e;
  for (int t = 1; t < T; t++) {
    const char *p = b + bytes * t / T;
    if (p < cut[t - 1]) p = cut[t - 1];
    const char *nl = (const char *)std::memchr(p, '\n', (size_t)(e - p));
    cut[t] = nl ? nl + 1 : e;
  }
  std::vector<std::vector<double>> part(T);
  std::vector<int> ok(T, 1);
  auto work = [&](int t) {
    part[t].reserve((size_t)(cut[t + 1] - cut[t]) / 20 + 16);
    for_lines(cut[t], cut[t + 1], [&](const char *lb, const char *le) {
      if (ok[t] && !parse_csv_line(lb, le, part[t])) ok[t] = 0;
    });
  };
  if (T == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < T; t++) th.emplace_back(work, t);
    for (auto &x : th) x.join();
  }
  size_t n = 0;
  for (int t = 0; t < T; t++) {
    if (!ok[t]) return GWGPU_EINVAL;
    n += part[t].size();
  }
  out.reserve(out.size() + n);
  for (int t = 0; t < T; t++) out.insert(out.end(), part[t].begin(), part[t].end());
  return GWGPU_OK;
}

// White-space separated tokens of [b, e) (istringstream >> std::string).
template <class F>
bool for_tokens(const char *b, const char *e, F &&fn) {
  while (b < e) {
    while (b < e && std::isspace((unsigned char)*b)) b++;
    if (b >= e) break;
    const char *t = b;
    while (b < e && !std::isspace((unsigned char)*b)) b++;
    if (!fn(t, b)) return false;
  }
  return true;
}

// read_LOSC_data_file (io_util.cpp:403-464).  Line 0 is skipped; in line 1
// every token that starts with a digit sets fs; in line 2 the first such token
// is the GPS start time and later ones the duration; from line 3 on, the
// comma-separated values are the strain samples.
int read_losc_data(const char *path, std::vector<double> &samples, double *start, double *duration, double *fs) {
  std::string s;
  if (!path || !read_whole(path, s)) return GWGPU_ENOTFOUND;
  const char *b = s.data(), *e = b + s.size();
  int j = 0;
  const char *body = e;
  bool bad = false;
  while (b < e && j < 3) {
    const char *nl = (const char *)std::memchr(b, '\n', (size_t)(e - b));
    const char *le = nl ? nl : e;
    if (j == 1) {
      for_tokens(b, le, [&](const char *t, const char *te) {
        if (std::isdigit((unsigned char)*t) && !parse_double(t, te, fs)) bad = true;
        return true;
      });
    } else if (j == 2) {
      int k = 0;
      for_tokens(b, le, [&](const char *t, const char *te) {
        if (std::isdigit((unsigned char)*t)) {
          if (!parse_double(t, te, k == 0 ? start : duration)) bad = true;
          k = 1;
        }
        return true;
      });
    }
    j++;
    b = nl ? nl + 1 : e;
    body = b;
  }
  if (bad) return GWGPU_EINVAL;
  samples.clear();
  return parse_csv_block(body, e, samples);
}

// read_LOSC_PSD_file (io_util.cpp:466-500): the first line skipped, then
// white-space separated values, row-major rows x cols.
int read_losc_psd(const char *path, double *out, int rows, int cols) {
  std::string s;
  if (!path || !read_whole(path, s)) return GWGPU_ENOTFOUND;
  const char *b = s.data(), *e = b + s.size();
  const char *nl = (const char *)std::memchr(b, '\n', (size_t)(e - b));
  b = nl ? nl + 1 : e;
  const size_t cap = (size_t)rows * cols;
  size_t i = 0;
  bool ok = for_tokens(b, e, [&](const char *t, const char *te) {
    double v;
    if (i >= cap || !parse_double(t, te, &v)) return false;
    out[i++] = v;
    return true;
  });
  if (!ok) return i >= cap ? GWGPU_ETOOLARGE : GWGPU_EINVAL;
  for (; i < cap; i++) out[i] = 0.0;  // rows beyond the file (the reference leaves them unset)
  return GWGPU_OK;
}

// ------------------------------------------------------------ noise curves
// aLIGO_analytic (detector_util.cpp:286-293): the amplitude spectral density.
double aligo_analytic(double f) {
  const double S = 3e-48, fknee = 70.;
  const double x = fknee / f, x4 = x * x * x * x;
  return std::sqrt(S * (x4 + 2 + 2 * x * x) / 5);
}

// Hanford_O1_fitted (detector_util.cpp:404-414): sqrt(S0) exp(sum_k a_k ln^k f).
double hanford_o1_fitted(double f) {
  const double a[7] = {47.8466, -92.1896, 35.9273, -7.61447, 0.916742, -0.0588089, 0.00156345};
  const double S0 = .8464, x = std::log(f);
  return std::sqrt(S0) * std::exp(a[0] + a[1] * x + a[2] * x * x + a[3] * x * x * x + a[4] * x * x * x * x +
                                  a[5] * x * x * x * x * x + a[6] * x * x * x * x * x * x);
}

// The tabulated curves by name and file (detector_util.cpp:164-241).  The
// two KAGRA "_smoothed" names are listed by the reference but have no file.
struct Curve {
  const char *name, *file;
};
const Curve kCurves[] = {
    {"AdLIGOMidHigh", "AdLIGOMidHigh.csv"},
    {"_AdLIGODesign", "AdLIGODesign.csv"},
    {"AdLIGODesign", "aligo_O4high.csv"},
    {"AdLIGODesign_smoothed", "aligo_O4high_smoothed.csv"},
    {"AdLIGOAPlus", "AplusDesign.csv"},
    {"AdLIGOAPlus_smoothed", "AplusDesign_smoothed.csv"},
    {"CE1", "CE1_strain.csv"},
    {"CE1_smoothed", "CE1_strain_smoothed.csv"},
    {"CE2", "CE2_strain.csv"},
    {"CE2_smoothed", "CE2_strain_smoothed.csv"},
    {"AdVIRGOPlus2_opt", "avirgo_O5high_NEW.csv"},
    {"AdVIRGOPlus2_opt_smoothed", "avirgo_O5high_NEW_smoothed.csv"},
    {"AdVIRGOPlus2_pess", "avirgo_O5low_NEW.csv"},
    {"AdVIRGOPlus2_pess_smoothed", "avirgo_O5low_NEW_smoothed.csv"},
    {"AdVIRGOPlus1", "avirgo_O4high_NEW.csv"},
    {"AdVIRGOPlus1_smoothed", "avirgo_O4high_NEW_smoothed.csv"},
    {"KAGRA_opt", "kagra_128Mpc.csv"},
    {"KAGRA_pess", "kagra_80Mpc.csv"},
    {"ET-D", "ET-0000A-18_ETDSensitivityCurveTxtFile.csv"},
    {"ET-D_smoothed", "ETDXylophoneDwyer.csv"},
    {"AdLIGOVoyager", "Voyager.csv"},
};

// Linear interpolation through (x_i, y_i) at f (gsl_interp_linear: the
// interval i with x_i <= f < x_{i+1}, the last interval at f = x_{n-1}); NaN
// outside [x_0, x_{n-1}].
double interp_linear(const std::vector<double> &x, const std::vector<double> &y, double f) {
  const size_t n = x.size();
  if (!(f >= x[0] && f <= x[n - 1])) return NAN;
  size_t lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    size_t mid = (lo + hi) / 2;
    if (x[mid] > f) hi = mid;
    else lo = mid;
  }
  const double dx = x[lo + 1] - x[lo];
  return y[lo] + (f - x[lo]) / dx * (y[lo + 1] - y[lo]);
}

// ----------------------------------------------------------- LOSC transform
constexpr int kBlock = 256;

// x[d][l] *= Tukey window w(l) for l < count (the rest of each row is zero).
// util.cpp:1736-1757: imin, imax truncated to integers; the taper
// 0.5 (1 + cos(pi (l / imin - 1))) below imin, 1 below imax, and
// 0.5 (1 + cos(pi (l / imin - 2 / alpha + 1))) from imax on.
__global__ void k_losc_window(double *__restrict__ x, int n_trim, int count, double imin, double imax,
                              double alpha) {
  const int d = blockIdx.y;
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < count; l += gridDim.x * blockDim.x) {
    double w;
    if (l < imin) w = 0.5 * (1 + cos(M_PI * ((double)l / imin - 1)));
    else if (l < imax) w = 1;
    else w = 0.5 * (1 + cos(M_PI * ((double)l / imin - 2. / alpha + 1.)));
    x[(size_t)d * n_trim + l] *= w;
  }
}

// out[d][l] = dt * X_d[k0 + l], from the half spectrum of the real transform
// (X[n - k] = conj(X[k]) above n/2).
__global__ void k_losc_select(const double2 *__restrict__ X, int n_trim, int k0, int nb, double dt,
                              double2 *__restrict__ out) {
  const int d = blockIdx.y, half = n_trim / 2 + 1;
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < nb; l += gridDim.x * blockDim.x) {
    const int k = k0 + l;
    double2 v;
    if (k < half) {
      v = X[(size_t)d * half + k];
    } else {
      v = X[(size_t)d * half + (n_trim - k)];
      v.y = -v.y;
    }
    out[(size_t)d * nb + l] = make_double2(dt * v.x, dt * v.y);
  }
}

// First index i in [lo, hi) with pred(i) true, for a predicate that is false
// then true along i (hi when never true).
template <class P>
long long first_true(long long lo, long long hi, P &&pred) {
  while (lo < hi) {
    long long mid = lo + (hi - lo) / 2;
    if (pred(mid)) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

int losc_prepare(gwgpu_context *c, const double *const *series, int nd, long long series_length, double file_start,
                 double duration, double fs, const double *tab, int psd_length, double trigger_time,
                 double post_merger_duration, double *data, double *psds, double *freqs, int *bins_out) {
  const int cols = nd + 1;
  // PSDs and frequencies straight from the table (io_util.cpp:557-562)
  for (int j = 0; j < psd_length; j++)
    for (int i = 0; i < nd; i++) {
      psds[(size_t)i * psd_length + j] = tab[(size_t)j * cols + i + 1];
      freqs[(size_t)i * psd_length + j] = tab[(size_t)j * cols];
    }
  const double Tobs = 1. / (tab[cols] - tab[0]);
  const double df = 1. / Tobs, dt = 1. / fs;
  const int n_trim = (int)(Tobs * fs);
  const long long N = (long long)(fs * duration);
  const double time_start = trigger_time - (Tobs - post_merger_duration);
  const double time_end = trigger_time + post_merger_duration;
  if (time_start < file_start || time_end > (file_start + duration)) {
    c->last_error = "trigger time does not fit inside the data file";
    return GWGPU_EDOMAIN;
  }
  if (n_trim < 2) {
    c->last_error = "observation time shorter than two samples";
    return GWGPU_EINVAL;
  }
  // samples with time_start < t_i <= time_end, t_i = file_start + i dt (contiguous in i)
  auto t_of = [&](long long i) { return file_start + i * dt; };
  const long long i0 = first_true(0, N, [&](long long i) { return t_of(i) > time_start; });
  const long long i1 = first_true(0, N, [&](long long i) { return t_of(i) > time_end; });
  long long count = std::max(0LL, i1 - i0);
  count = std::min<long long>(count, n_trim);  // the reference writes past its n_trim buffer here
  if (i0 + count > series_length) {
    c->last_error = "data file shorter than its header's duration";
    return GWGPU_EINVAL;
  }
  // frequency bins k df with fmin <= k df <= fmax (contiguous in k)
  const double fmin = tab[0], fmax = tab[(size_t)(psd_length - 1) * cols];
  const long long k0 = first_true(0, n_trim, [&](long long k) { return k * df >= fmin; });
  const long long k1 = first_true(k0, n_trim, [&](long long k) { return k * df > fmax; });
  const int nb = (int)std::min<long long>(std::max(0LL, k1 - k0), psd_length);
  const double alpha = 2 * .4 / Tobs;
  const double imin = (int)(alpha * (double)(n_trim - 1) / 2.0);
  const double imax = (int)((double)(n_trim - 1) * (1. - alpha / 2.));

  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  int plan;
  int st = gwfft::plan(c, gwfft::kD2Z, n_trim, nd, &plan);
  if (st) return st;
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t half = (size_t)n_trim / 2 + 1;
  const size_t o_x = 0, o_X = up(8 * (size_t)nd * n_trim), o_o = o_X + up(16 * (size_t)nd * half),
               total = o_o + up(16 * (size_t)nd * std::max(nb, 1));
  void *dev;
  if ((st = c->workspace(gwgpu_context::kWsIngest, total, &dev))) return st;
  char *b = (char *)dev;
  double *x = (double *)(b + o_x);
  double2 *X = (double2 *)(b + o_X), *o = (double2 *)(b + o_o);
  cudaMemsetAsync(x, 0, 8 * (size_t)nd * n_trim, c->stream);
  for (int d = 0; d < nd; d++)
    if (count)
      cudaMemcpyAsync(x + (size_t)d * n_trim, series[d] + i0, 8 * (size_t)count, cudaMemcpyHostToDevice, c->stream);
  const int gx = (int)std::min<long long>((std::max(count, 1LL) + kBlock - 1) / kBlock, 1024);
  if (count) k_losc_window<<<dim3(gx, nd), kBlock, 0, c->stream>>>(x, n_trim, (int)count, imin, imax, alpha);
  if ((st = gwfft::exec_d2z(c, plan, x, X, c->stream))) return st;
  if (nb) {
    const int gb = std::min((nb + kBlock - 1) / kBlock, 1024);
    k_losc_select<<<dim3(gb, nd), kBlock, 0, c->stream>>>(X, n_trim, (int)k0, nb, dt, o);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->fail(e, "strain transform launch");
  for (int d = 0; d < nd; d++) {
    if (nb)
      cudaMemcpyAsync(data + (size_t)d * 2 * psd_length, o + (size_t)d * nb, 16 * (size_t)nb, cudaMemcpyDeviceToHost,
                      c->stream);
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "strain transform");
  // bins the band did not fill (the reference leaves them unset)
  for (int d = 0; d < nd; d++)
    std::fill(data + (size_t)d * 2 * psd_length + 2 * (size_t)nb, data + (size_t)(d + 1) * 2 * psd_length, 0.0);
  if (bins_out) *bins_out = nb;
  return GWGPU_OK;
}

}  // namespace

extern "C" {

int gwgpu_count_lines_data_file(const char *path, int *count) {
  std::string s;
  if (!count) return GWGPU_EINVAL;
  if (!path || !read_whole(path, s)) return GWGPU_ENOTFOUND;
  *count = (int)count_lines(s);
  return GWGPU_OK;
}

int gwgpu_count_lines_losc_data_file(const char *path, int *count) {
  int st = gwgpu_count_lines_data_file(path, count);
  if (st == GWGPU_OK) *count -= 3;
  return st;
}

int gwgpu_count_lines_losc_psd_file(const char *path, int *count) {
  int st = gwgpu_count_lines_data_file(path, count);
  if (st == GWGPU_OK) *count -= 1;
  return st;
}

int gwgpu_read_losc_data_file(const char *path, double *output, long long capacity, long long *count,
                              double *data_start_time, double *duration, double *fs) {
  if (!output || !data_start_time || !duration || !fs) return GWGPU_EINVAL;
  std::vector<double> v;
  int st = read_losc_data(path, v, data_start_time, duration, fs);
  if (st) return st;
  if (count) *count = (long long)v.size();
  if ((long long)v.size() > capacity) return GWGPU_ETOOLARGE;
  std::copy(v.begin(), v.end(), output);
  return GWGPU_OK;
}

int gwgpu_read_losc_psd_file(const char *path, double *output, int rows, int cols) {
  if (!output || rows < 1 || cols < 1) return GWGPU_EINVAL;
  return read_losc_psd(path, output, rows, cols);
}

int gwgpu_populate_noise(const double *frequencies, const char *detector, double *noise_root, int length,
                         double integration_time, const char *noise_dir) {
  (void)integration_time;  // only the LISA confusion-noise curves use it
  if (!frequencies || !detector || !noise_root || length < 0) return GWGPU_EINVAL;
  const std::string det(detector);
  if (det == "aLIGO_analytic" || det == "Hanford_O1_fitted") {
    for (int i = 0; i < length; i++)
      noise_root[i] = det == "aLIGO_analytic" ? aligo_analytic(frequencies[i]) : hanford_o1_fitted(frequencies[i]);
    return GWGPU_OK;
  }
  const char *file = nullptr;
  for (const Curve &cv : kCurves)
    if (det == cv.name) file = cv.file;
  if (!file || !noise_dir) return file ? GWGPU_EINVAL : GWGPU_ENOTFOUND;
  std::string path = std::string(noise_dir);
  if (!path.empty() && path.back() != '/') path += '/';
  path += file;
  std::string s;
  if (!read_whole(path.c_str(), s)) return GWGPU_ENOTFOUND;
  std::vector<double> v;
  int st = parse_csv_block(s.data(), s.data() + s.size(), v);
  if (st) return st;
  // read_file(.., rows, 2) with rows = the file's line count: the values in
  // order, two per row (blank lines carry none)
  const size_t rows = v.size() / 2;
  if (rows < 2) return GWGPU_EINVAL;
  std::vector<double> x(rows), y(rows);
  for (size_t i = 0; i < rows; i++) {
    x[i] = v[2 * i];
    y[i] = v[2 * i + 1];
  }
  for (size_t i = 1; i < rows; i++)
    if (!(x[i] > x[i - 1])) return GWGPU_EINVAL;  // gsl_spline_init needs increasing abscissae
  bool outside = false;
  for (int i = 0; i < length; i++) {
    noise_root[i] = interp_linear(x, y, frequencies[i]);
    if (std::isnan(noise_root[i])) outside = true;
  }
  return outside ? GWGPU_EDOMAIN : GWGPU_OK;
}

int gwgpu_losc_prepare(gwgpu_context *c, const double *series, int num_detectors, long long series_length,
                       double file_start, double duration, double fs, const double *psd_table, int psd_length,
                       double trigger_time, double post_merger_duration, double *data, double *psds, double *freqs,
                       int *bins_out) {
  if (!c || !series || num_detectors < 1 || series_length < 1 || !psd_table || psd_length < 2 || !data || !psds ||
      !freqs || !(fs > 0) || !(duration > 0))
    return GWGPU_EINVAL;
  std::vector<const double *> rows(num_detectors);
  for (int d = 0; d < num_detectors; d++) rows[d] = series + (size_t)d * series_length;
  return losc_prepare(c, rows.data(), num_detectors, series_length, file_start, duration, fs, psd_table, psd_length,
                      trigger_time, post_merger_duration, data, psds, freqs, bins_out);
}

int gwgpu_allocate_losc_data(gwgpu_context *c, const char *const *data_files, const char *psd_file,
                             int num_detectors, int psd_length, int data_file_length, double trigger_time,
                             double post_merger_duration, double *data, double *psds, double *freqs) {
  if (!c || !data_files || !psd_file || num_detectors < 1 || psd_length < 2 || data_file_length < 1 || !data ||
      !psds || !freqs)
    return GWGPU_EINVAL;
  // the detectors' files in parallel; the header of the last one is kept
  // (io_util.cpp:537-539)
  std::vector<std::vector<double>> s(num_detectors);
  std::vector<double> st0(num_detectors), dur(num_detectors), fsv(num_detectors);
  std::vector<int> rc(num_detectors, GWGPU_OK);
  {
    std::vector<std::thread> th;
    for (int d = 0; d < num_detectors; d++)
      th.emplace_back([&, d] { rc[d] = read_losc_data(data_files[d], s[d], &st0[d], &dur[d], &fsv[d]); });
    for (auto &t : th) t.join();
  }
  for (int d = 0; d < num_detectors; d++) {
    if (rc[d]) {
      c->last_error = std::string("reading ") + (data_files[d] ? data_files[d] : "(null)");
      return rc[d];
    }
    if ((long long)s[d].size() > data_file_length) return GWGPU_ETOOLARGE;
    s[d].resize(data_file_length, 0.0);
  }
  std::vector<double> tab((size_t)psd_length * (num_detectors + 1));
  int st = read_losc_psd(psd_file, tab.data(), psd_length, num_detectors + 1);
  if (st) {
    c->last_error = std::string("reading ") + psd_file;
    return st;
  }
  std::vector<const double *> rows(num_detectors);
  for (int d = 0; d < num_detectors; d++) rows[d] = s[d].data();
  const int last = num_detectors - 1;
  return losc_prepare(c, rows.data(), num_detectors, data_file_length, st0[last], dur[last], fsv[last], tab.data(),
                      psd_length, trigger_time, post_merger_duration, data, psds, freqs, nullptr);
}

}  // extern "C"
