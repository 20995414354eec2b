// bsglmm_main.cpp -- the `bsglmm` command: a BinCar-compatible driver in
// C++ over the C ABI of libbsglmm_gb300.so.
//
//   bsglmm NTypes NCov GPU Design Mask WM [MaxIter BurnIn]
//
// Same arguments, inputs and outputs as the reference program (main.cu:60-183
// argv and set-up, read_data.cpp:187-545 inputs, mcmc.cpp:795-975 outputs):
//   Mask    a FLOAT64 NIfTI-1 image in ./images ("1": images/mask.nii.gz);
//           voxels whose value converts to a nonzero byte are in the mask
//   Design  a header of NCov+2 tokens, then per subject: id, NCov covariates,
//           lesion-map file name relative to ./images (FLOAT32/FLOAT64 NIfTI,
//           binary); the first NTypes covariates are the group columns
//   WM      "0" none, "1" images/avg152T1_white.nii.gz, else a UINT8 image in
//           ./images; WM_v = value / 255 and beta_WM is drawn every sweep
//   seed.dat  three integers (KISS state), advanced and rewritten at exit
// Outputs (FLOAT64 NIfTI-1, gzipped in process): empir_prb_<group>,
// total_lesion_cnt, total_empir_prb, spatCoef_<cov>, spatCoef_<cov>.Var,
// standCoef_<cov>, prb_<group>, bWM (with a WM image); Qhat.dat, Qhat2.dat
// and DIC.dat from the predictive pass run after every kept sweep.  Every
// segment of up to 100 sweeps also prints one JSON line on stderr: the
// sweep range, device milliseconds per sweep and subject-voxel updates/s.
//
// The chain runs MaxIter+1 sweeps with the reference's burn-in and SAVE_ITER
// thinning (mcmc.cpp:303-308) and the reference GPU path's Wishart df
// V + 19 (covarGPU.cu:1104).  It is the C++ form of bsglmm_gb300/driver.py
// and writes the same files.  Exit status: 0 ok, 1 usage, 2 input error,
// 3 sampler error.
#include <dlfcn.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/bsglmm_gb300.h"

namespace {

struct InputError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct SamplerError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

const char *kUsage =
    "Usage: bsglmm  NTypes  NCov  GPU  Design Mask WM [MaxIter BurnIn]\n"
    "  NTypes  - Number of groups\n"
    "  NCov    - Number of covariates (count must include groups)\n"
    "  GPU     - 1 use GPU (this build has no CPU path)\n"
    "  Design  - Text file, tab or space separated data file\n"
    "  Mask    - Filename of mask image in './images' directory, or '1' to use default "
    "(mask.nii.gz)\n"
    "  WM      - Filename of WM image in './images' directory, '0' to use none, or '1' to "
    "use default (avg152T1_white.nii.gz)\n"
    "  MaxIter - Number of iterations (defaults to 100,000)\n"
    "  BurnIn  - Number of burn-in iterations (defaults to 50,000)\n";

// ------------------------------------------------------ gzip via zlib ----
// zlib is opened at run time (libz.so.1), so the build needs no zlib
// headers; the four gz* calls have a stable C ABI.
struct Zlib {
  void *h = nullptr;
  void *(*gzopen)(const char *, const char *) = nullptr;
  int (*gzread)(void *, void *, unsigned) = nullptr;
  int (*gzwrite)(void *, const void *, unsigned) = nullptr;
  int (*gzclose)(void *) = nullptr;
  Zlib() {
    h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("libz.so", RTLD_NOW | RTLD_LOCAL);
    if (!h) return;
    gzopen = reinterpret_cast<void *(*)(const char *, const char *)>(dlsym(h, "gzopen"));
    gzread = reinterpret_cast<int (*)(void *, void *, unsigned)>(dlsym(h, "gzread"));
    gzwrite = reinterpret_cast<int (*)(void *, const void *, unsigned)>(dlsym(h, "gzwrite"));
    gzclose = reinterpret_cast<int (*)(void *)>(dlsym(h, "gzclose"));
  }
  bool ok() const { return gzopen && gzread && gzwrite && gzclose; }
};

Zlib &zlib() {
  static Zlib z;
  return z;
}

// The whole file, gunzipped when it starts with the gzip magic.
std::vector<unsigned char> read_file(const std::string &path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw InputError(path + ": no such file");
  std::vector<unsigned char> raw((std::istreambuf_iterator<char>(f)),
                                 std::istreambuf_iterator<char>());
  if (raw.size() < 2 || raw[0] != 0x1f || raw[1] != 0x8b) return raw;
  Zlib &z = zlib();
  if (!z.ok()) throw InputError(path + ": gzip-compressed and zlib is not available");
  void *gz = z.gzopen(path.c_str(), "rb");
  if (!gz) throw InputError(path + ": cannot open");
  std::vector<unsigned char> out;
  unsigned char buf[1 << 16];
  int n;
  while ((n = z.gzread(gz, buf, sizeof(buf))) > 0) out.insert(out.end(), buf, buf + n);
  z.gzclose(gz);
  if (n < 0) throw InputError(path + ": corrupt gzip stream");
  return out;
}

// ------------------------------------------------------------- NIfTI-1 ----
enum { UINT8 = 2, INT16 = 4, INT32 = 8, FLOAT32 = 16, FLOAT64 = 64, INT8 = 256,
       UINT16 = 512, UINT32 = 768, INT64 = 1024, UINT64 = 1280 };

struct Image {
  int X = 0, Y = 0, Z = 0, datatype = 0;
  std::vector<double> data;  // x fastest
};

template <typename T>
T load(const unsigned char *p, bool swap) {
  unsigned char b[sizeof(T)];
  std::memcpy(b, p, sizeof(T));
  if (swap)
    for (size_t i = 0; i < sizeof(T) / 2; ++i) std::swap(b[i], b[sizeof(T) - 1 - i]);
  T v;
  std::memcpy(&v, b, sizeof(T));
  return v;
}

// A single-file NIfTI-1 image (348-byte header, data at vox_offset >= 352),
// either byte order, as read_data.cpp:187-247 reads one after gunzip.
Image read_nifti(const std::string &path) {
  std::vector<unsigned char> raw = read_file(path);
  if (raw.size() < 348) throw InputError(path + ": shorter than a NIfTI-1 header");
  bool swap = false;
  if (load<int32_t>(raw.data(), false) != 348) {
    if (load<int32_t>(raw.data(), true) != 348)
      throw InputError(path + ": not a NIfTI-1 file (sizeof_hdr != 348)");
    swap = true;
  }
  int16_t dim[8];
  for (int i = 0; i < 8; ++i) dim[i] = load<int16_t>(raw.data() + 40 + 2 * i, swap);
  Image im;
  im.datatype = load<int16_t>(raw.data() + 70, swap);
  const float vox_offset = load<float>(raw.data() + 108, swap);
  if (std::memcmp(raw.data() + 344, "n+1", 3) != 0)
    throw InputError(path + ": not a single-file NIfTI-1 image");
  if (dim[0] < 3 || dim[1] < 1 || dim[2] < 1 || dim[3] < 1)
    throw InputError(path + ": bad dimensions");
  im.X = dim[1];
  im.Y = dim[2];
  im.Z = dim[3];
  size_t esize = 0;
  switch (im.datatype) {
    case UINT8: case INT8: esize = 1; break;
    case INT16: case UINT16: esize = 2; break;
    case INT32: case UINT32: case FLOAT32: esize = 4; break;
    case FLOAT64: case INT64: case UINT64: esize = 8; break;
    default: throw InputError(path + ": unsupported datatype " + std::to_string(im.datatype));
  }
  const size_t n = (size_t)im.X * im.Y * im.Z;
  const size_t off = std::max<size_t>((size_t)vox_offset, 352);
  if (raw.size() < off + n * esize) throw InputError(path + ": truncated image data");
  im.data.resize(n);
  const unsigned char *p = raw.data() + off;
  for (size_t i = 0; i < n; ++i, p += esize) {
    double v = 0;
    switch (im.datatype) {
      case UINT8: v = p[0]; break;
      case INT8: v = (int8_t)p[0]; break;
      case INT16: v = load<int16_t>(p, swap); break;
      case UINT16: v = load<uint16_t>(p, swap); break;
      case INT32: v = load<int32_t>(p, swap); break;
      case UINT32: v = load<uint32_t>(p, swap); break;
      case FLOAT32: v = load<float>(p, swap); break;
      case FLOAT64: v = load<double>(p, swap); break;
      case INT64: v = (double)load<int64_t>(p, swap); break;
      case UINT64: v = (double)load<uint64_t>(p, swap); break;
    }
    im.data[i] = v;
  }
  return im;
}

void put32(std::vector<unsigned char> &h, size_t at, const void *v, size_t n) {
  std::memcpy(h.data() + at, v, n);
}

// FLOAT64, 2 mm voxels, vox_offset 352, mm units, magic "n+1" -- the image
// the reference writes (nifti1_read_write.cpp:229-254) -- gzipped in process.
void write_nifti_gz(const std::string &path, const std::vector<double> &data, int X, int Y,
                    int Z) {
  std::vector<unsigned char> blob(352, 0);
  const int32_t sizeof_hdr = 348;
  put32(blob, 0, &sizeof_hdr, 4);
  const int16_t dim[8] = {3, (int16_t)X, (int16_t)Y, (int16_t)Z, 1, 0, 0, 0};
  put32(blob, 40, dim, 16);
  const int16_t dt[2] = {FLOAT64, 64};
  put32(blob, 70, dt, 4);
  const float pixdim[8] = {0.f, 2.f, 2.f, 2.f, 0.f, 0.f, 0.f, 0.f};
  put32(blob, 76, pixdim, 32);
  const float vox_offset = 352.f;
  put32(blob, 108, &vox_offset, 4);
  blob[123] = 2;  // NIFTI_UNITS_MM
  std::memcpy(blob.data() + 344, "n+1\0", 4);
  const size_t n = (size_t)X * Y * Z;
  if (data.size() != n) throw InputError(path + ": data size does not match the dimensions");
  const unsigned char *d = reinterpret_cast<const unsigned char *>(data.data());
  blob.insert(blob.end(), d, d + n * sizeof(double));
  Zlib &z = zlib();
  if (!z.ok()) throw InputError(path + ": zlib is not available to gzip the output");
  void *gz = z.gzopen(path.c_str(), "wb6");
  if (!gz) throw InputError(path + ": cannot write");
  size_t done = 0;
  while (done < blob.size()) {
    const unsigned chunk = (unsigned)std::min<size_t>(blob.size() - done, 1u << 30);
    if (z.gzwrite(gz, blob.data() + done, chunk) != (int)chunk) {
      z.gzclose(gz);
      throw InputError(path + ": write failed");
    }
    done += chunk;
  }
  if (z.gzclose(gz) != 0) throw InputError(path + ": write failed");
}

// C's (unsigned char) conversion of a double (read_data.cpp:235,385).
uint8_t as_byte(double v) {
  if (!std::isfinite(v)) return 0;
  double t = std::trunc(v);
  if (t > 9.2e18 || t < -9.2e18) return 0;
  int64_t i = (int64_t)t % 256;
  return (uint8_t)(i < 0 ? i + 256 : i);
}

// --------------------------------------------------------------- inputs ----
struct Design {
  std::vector<std::string> names;
  std::vector<float> covar;  // [P][N]
  std::vector<std::string> images;
  int N = 0;
};

Design read_design(const std::string &path, int ncov) {
  std::ifstream f(path);
  if (!f) throw InputError(path + ": no such file");
  std::vector<std::string> tok;
  std::string t;
  while (f >> t) tok.push_back(t);
  const size_t width = (size_t)ncov + 2;
  if (tok.size() < width) throw InputError(path + ": header needs " + std::to_string(width) +
                                           " tokens");
  Design d;
  for (int p = 0; p < ncov; ++p) d.names.push_back(tok[1 + p]);
  const size_t body = tok.size() - width;
  if (body == 0 || body % width)
    throw InputError(path + ": " + std::to_string(body) +
                     " tokens after the header is not a multiple of NCov+2 = " +
                     std::to_string(width));
  d.N = (int)(body / width);
  d.covar.assign((size_t)ncov * d.N, 0.f);
  for (int i = 0; i < d.N; ++i) {
    const std::string *row = &tok[width + (size_t)i * width];
    for (int p = 0; p < ncov; ++p) {
      char *end = nullptr;
      const double v = std::strtod(row[1 + p].c_str(), &end);
      if (!end || *end) throw InputError(path + ": non-numeric covariate " + row[1 + p]);
      d.covar[(size_t)p * d.N + i] = (float)v;
    }
    d.images.push_back("images/" + row[ncov + 1]);
  }
  return d;
}

// ------------------------------------------------------------------ KISS --
// The KISS step of randgen.cpp:9-23 (64-bit words, 2^-64 scale).
double kiss(uint64_t s[3]) {
  s[1] = s[1] ^ (s[1] << 17);
  s[2] = (s[2] ^ (s[2] << 18)) & 0x7FFFFFFFull;
  s[0] = 69069ull * s[0] + 23606797ull;
  s[1] ^= s[1] >> 15;
  s[2] ^= s[2] >> 13;
  return (double)(uint64_t)(s[0] + s[1] + s[2]) * 5.421010862427522e-20;
}

// The chain's 64-bit Philox key from two draws of the seed's KISS stream
// (the stream advances, so seed.dat changes from run to run as in the
// reference).
uint64_t chain_key(uint64_t s[3]) {
  const uint64_t hi = (uint64_t)(kiss(s) * 4294967296.0);
  const uint64_t lo = (uint64_t)(kiss(s) * 4294967296.0);
  return (hi << 32) ^ lo;
}

int save_iter_rule(int maxiter, int burnin) {  // mcmc.cpp:303-308
  if (maxiter - burnin < 10000) return std::max(1, maxiter - burnin);
  return (maxiter - burnin) / 10000;
}

// ----------------------------------------------------------------- run ----
void check(bsg_ctx *ctx, bsg_status s, const char *where) {
  if (s != BSG_OK) {
    std::string m = std::string(where) + ": " + bsg_status_string(s);
    const char *d = bsg_last_error(ctx);
    if (d && *d) m += std::string(" (") + d + ")";
    throw SamplerError(m);
  }
}

// Inverse of a small SPD matrix by Gauss-Jordan elimination with partial
// pivoting (for the periodic summary only).
std::vector<double> inverse(std::vector<double> a, int n) {
  std::vector<double> inv((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) inv[i + i * n] = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[c + r * n]) > std::fabs(a[c + piv * n])) piv = r;
    for (int k = 0; k < n; ++k) {
      std::swap(a[k + c * n], a[k + piv * n]);
      std::swap(inv[k + c * n], inv[k + piv * n]);
    }
    const double d = a[c + c * n];
    for (int k = 0; k < n; ++k) {
      a[k + c * n] /= d;
      inv[k + c * n] /= d;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = a[c + r * n];
      for (int k = 0; k < n; ++k) {
        a[k + r * n] -= f * a[k + c * n];
        inv[k + r * n] -= f * inv[k + c * n];
      }
    }
  }
  return inv;
}

// The periodic summary of mcmc.cpp:535-583.
void print_state(int it, const std::vector<double> &omega, const std::vector<float> &colmean,
                 int P, int ntypes) {
  const std::vector<double> V = inverse(omega, P);
  std::vector<double> sd(P);
  for (int i = 0; i < P; ++i) sd[i] = std::sqrt(V[i + i * P]);
  std::printf("iter = %d\t\n  overall mean and SD for groups \n", it);
  for (int i = 0; i < ntypes; ++i) std::printf("\t %10.6f %10.6f\n", colmean[i], sd[i]);
  std::printf("\n  overall mean and SD for spatially varying coefficients for all covariates \n");
  for (int i = ntypes; i < P; ++i) std::printf("\t %10.6f %10.6f\n", colmean[i], sd[i]);
  std::printf("\n  correlation matrix of regression parameters \n");
  for (int i = 0; i < P; ++i) {
    for (int j = 0; j <= i; ++j) std::printf("   %6.3f ", V[j + i * P] / (sd[i] * sd[j]));
    std::printf("\n");
  }
  std::printf("\n");
  std::fflush(stdout);
}

// Rows of Qhat.dat / Qhat2.dat (mcmc.cpp:719-786): subject, the normalised
// exp(Qhat), the predicted group (last maximum) and the true group (first
// nonzero group column, else 0); with prior, Qhat is first scaled by it.
std::string qhat_lines(const std::vector<double> &qhat, const std::vector<float> &covar, int N,
                       int S, int ntypes, const std::vector<double> *prior) {
  std::string out;
  char buf[64];
  for (int i = 0; i < N; ++i) {
    std::vector<double> q(S);
    for (int g = 0; g < S; ++g) q[g] = qhat[(size_t)i * S + g] * (prior ? (*prior)[g] : 1.0);
    double mx = -std::numeric_limits<double>::max();
    for (int g = 0; g < ntypes; ++g) mx = std::max(mx, q[g]);
    double s = 0;
    for (int g = 0; g < ntypes; ++g) s += std::exp(q[g] - mx);
    const double qh = std::log(s) + mx;
    std::snprintf(buf, sizeof(buf), "%d ", i);
    out += buf;
    for (int g = 0; g < ntypes; ++g) {
      std::snprintf(buf, sizeof(buf), "%.6f ", std::exp(q[g] - qh));
      out += buf;
    }
    mx = -std::numeric_limits<double>::max();
    int pred = -1, truth = 0;
    for (int g = 0; g < ntypes; ++g)
      if (mx <= q[g]) {
        mx = q[g];
        pred = g;
      }
    for (int g = 0; g < ntypes; ++g)
      if (covar[(size_t)g * N + i] != 0.f) {
        truth = g;
        break;
      }
    std::snprintf(buf, sizeof(buf), "%d %d\n", pred, truth);
    out += buf;
  }
  return out;
}

void write_text(const std::string &path, const std::string &text) {
  std::ofstream f(path, std::ios::binary);
  if (!f) throw InputError(path + ": cannot write");
  f << text;
}

int run(int ntypes, int ncov, const std::string &design_path, const std::string &mask_name,
        const std::string &wm_name, int maxiter, int burnin) {
  Image mimg = read_nifti("images/" + mask_name);
  if (mimg.datatype != FLOAT64)
    throw InputError("Incorrect data type in file: " + std::to_string(mimg.datatype) +
                     "\nMust be float (NIFTI_TYPE_FLOAT64)");
  const int X = mimg.X, Y = mimg.Y, Z = mimg.Z;
  const size_t R = (size_t)X * Y * Z;
  std::vector<uint8_t> mask(R);
  for (size_t i = 0; i < R; ++i) mask[i] = as_byte(mimg.data[i]) != 0;
  std::vector<float> wm;
  if (!wm_name.empty()) {  // read_nifti1_WM (read_data.cpp:489-545)
    Image w = read_nifti("images/" + wm_name);
    if (w.datatype != UINT8)
      throw InputError("Incorrect data type in file: " + std::to_string(w.datatype) +
                       "\nMust be unsigned char (NIFTI_TYPE_UINT8)");
    if (w.X != X || w.Y != Y || w.Z != Z)
      throw InputError("images/" + wm_name + ": dimensions differ from the mask's");
    for (size_t i = 0; i < R; ++i)
      if (mask[i]) wm.push_back((float)w.data[i] / 255.0f);
  }
  Design d = read_design(design_path, ncov);
  if (ntypes > ncov) throw InputError("NTypes cannot exceed NCov");
  const int N = d.N;
  size_t V = 0;
  for (size_t i = 0; i < R; ++i) V += mask[i];
  std::vector<uint8_t> data((size_t)N * V);  // read_data.cpp:341-406
  std::fprintf(stderr, "Loading images: ");
  for (int i = 0; i < N; ++i) {
    Image im = read_nifti(d.images[i]);
    if (im.datatype != FLOAT32 && im.datatype != FLOAT64)
      throw InputError("Incorrect data type in file " + d.images[i] + ": " +
                       std::to_string(im.datatype) +
                       "\nMust be float (NIFTI_TYPE_FLOAT32) or double (NIFTI_TYPE_FLOAT64)");
    if (im.X != X || im.Y != Y || im.Z != Z)
      throw InputError(d.images[i] + ": dimensions differ from the mask's");
    size_t v = 0;
    for (size_t q = 0; q < R; ++q)
      if (mask[q]) {
        const uint8_t b = as_byte(im.data[q]);
        if (b > 1) throw InputError("lesion maps must be binary (0/1)");
        data[(size_t)i * V + v++] = b;
      }
    std::fprintf(stderr, ".");
  }
  std::fprintf(stderr, "\n");

  // write_empir_prb (read_data.cpp:418-487)
  std::vector<double> sum2(R, 0.0);
  for (int g = 0; g < ntypes; ++g) {
    std::vector<double> cnt(V, 0.0), full(R, 0.0);
    double members = 0;
    for (int i = 0; i < N; ++i)
      if (d.covar[(size_t)g * N + i] != 0.f) {
        members += 1;
        for (size_t v = 0; v < V; ++v) cnt[v] += data[(size_t)i * V + v];
      }
    size_t v = 0;
    for (size_t q = 0; q < R; ++q)
      if (mask[q]) {
        full[q] = cnt[v] / members;
        sum2[q] += cnt[v];
        ++v;
      }
    write_nifti_gz("empir_prb_" + d.names[g] + ".nii.gz", full, X, Y, Z);
  }
  write_nifti_gz("total_lesion_cnt.nii.gz", sum2, X, Y, Z);
  std::vector<double> total_p(R);
  for (size_t q = 0; q < R; ++q) total_p[q] = sum2[q] / N;
  write_nifti_gz("total_empir_prb.nii.gz", total_p, X, Y, Z);

  // seed.dat (main.cu:154-166)
  uint64_t seed[3] = {1, 2, 2};
  {
    std::ifstream sf("seed.dat");
    if (sf) {
      long long a, b, c;
      if (!(sf >> a >> b >> c)) throw InputError("seed.dat must hold three integers");
      seed[0] = (uint64_t)a;
      seed[1] = (uint64_t)b;
      seed[2] = (uint64_t)c;
    } else {
      std::printf("No seed.dat found; using [ 1 2 3 ]\n");
    }
  }
  const uint64_t key = chain_key(seed);

  bsg_ctx *ctx = nullptr;
  check(nullptr, bsg_create(0, &ctx), "bsg_create");
  struct Guard {
    bsg_ctx *c;
    ~Guard() { bsg_destroy(c); }
  } guard{ctx};
  bsg_dataset_desc dd{};
  dd.nrow = X;
  dd.ncol = Y;
  dd.ndepth = Z;
  dd.nsubs = N;
  dd.ncovar = ncov;
  dd.nsubtypes = ntypes;
  dd.mask = mask.data();
  dd.covar = d.covar.data();
  dd.data = data.data();
  dd.wm = wm.empty() ? nullptr : wm.data();
  int32_t ds = 0, ch = 0;
  check(ctx, bsg_add_dataset(ctx, &dd, &ds), "bsg_add_dataset");
  bsg_chain_desc cd{};
  cd.seed = key;
  cd.df_offset = 19;
  cd.burnin = burnin;
  cd.thin = save_iter_rule(maxiter, burnin);
  cd.beta_wm = 0.f;
  check(ctx, bsg_add_chain(ctx, ds, &cd, &ch), "bsg_add_chain");
  if (!wm.empty()) check(ctx, bsg_set_wm_update(ctx, ch, 1), "bsg_set_wm_update");
  if (ntypes >= 1) check(ctx, bsg_set_predictive(ctx, ch, 1), "bsg_set_predictive");
  const int P = ncov, S = ntypes;
  std::vector<double> omega((size_t)P * P);
  std::vector<float> colmean(P);
  const int kPrintEvery = 100;  // mcmc.cpp:309
  for (int done = 0; done <= maxiter;) {
    const int step = std::min(kPrintEvery, maxiter + 1 - done);
    if (done % kPrintEvery == 0) {
      check(ctx, bsg_get_omega(ctx, ch, omega.data()), "bsg_get_omega");
      check(ctx, bsg_get_colmeans(ctx, ch, colmean.data()), "bsg_get_colmeans");
      print_state(done, omega, colmean, P, ntypes);
    }
    double ms = 0.0;
    check(ctx, bsg_run_timed(ctx, step, &ms), "bsg_run_timed");
    check(ctx, bsg_sync(ctx), "bsg_sync");
    // one machine-readable line per segment on stderr
    std::fprintf(stderr,
                 "{\"sweeps\": [%d, %d], \"ms_per_sweep\": %.6g, "
                 "\"updates_per_s\": %.6g, \"status\": 0}\n",
                 done, done + step - 1, ms / step,
                 (double)N * (double)V * step / (ms > 0 ? ms * 1e-3 : 1e-300));
    done += step;
  }
  std::vector<double> sc((size_t)P * R), var((size_t)P * R), st((size_t)P * R),
      prb((size_t)std::max(S, 1) * R);
  check(ctx, bsg_get_maps(ctx, ch, sc.data(), var.data(), st.data(), prb.data()),
        "bsg_get_maps");
  int64_t nsw = 0, totsav = 0;
  check(ctx, bsg_get_sweep(ctx, ch, &nsw, &totsav), "bsg_get_sweep");
  std::printf("TOTSAV = %lld\n", (long long)totsav);
  double dic[4] = {NAN, NAN, NAN, NAN};
  if (S >= 1) {
    std::vector<double> qhat((size_t)N * S);
    double ed = 0;
    int64_t npred = 0;
    check(ctx, bsg_get_predictive(ctx, ch, qhat.data(), &ed, &npred), "bsg_get_predictive");
    write_text("Qhat.dat", qhat_lines(qhat, d.covar, N, S, ntypes, nullptr));
    std::vector<double> prior(S, 0.0);  // grp_prior (read_data.cpp:287-316)
    for (int g = 0; g < S; ++g) {
      for (int i = 0; i < N; ++i) prior[g] += std::trunc((double)d.covar[(size_t)g * N + i]);
      prior[g] /= N;
    }
    write_text("Qhat2.dat", qhat_lines(qhat, d.covar, N, S, ntypes, &prior));
    if (npred > 0) check(ctx, bsg_get_dic(ctx, ch, dic), "bsg_get_dic");
  }
  float bwm_now = 0.f;
  double bwm_mean = 0.0;
  check(ctx, bsg_get_beta_wm(ctx, ch, &bwm_now, &bwm_mean), "bsg_get_beta_wm");
  auto slab = [&](const std::vector<double> &a, int k) {
    return std::vector<double>(a.begin() + (size_t)k * R, a.begin() + (size_t)(k + 1) * R);
  };
  for (int p = 0; p < P; ++p) {
    write_nifti_gz("spatCoef_" + d.names[p] + ".nii.gz", slab(sc, p), X, Y, Z);
    write_nifti_gz("spatCoef_" + d.names[p] + ".Var.nii.gz", slab(var, p), X, Y, Z);
    write_nifti_gz("standCoef_" + d.names[p] + ".nii.gz", slab(st, p), X, Y, Z);
  }
  for (int g = 0; g < ntypes; ++g)
    write_nifti_gz("prb_" + d.names[g] + ".nii.gz", slab(prb, g), X, Y, Z);
  if (!wm.empty()) {  // mean over kept sweeps of beta_WM WM_v (mcmc.cpp:636,799)
    std::vector<double> b(R, 0.0);
    size_t v = 0;
    for (size_t q = 0; q < R; ++q)
      if (mask[q]) b[q] = bwm_mean * (double)wm[v++];
    write_nifti_gz("bWM.nii.gz", b, X, Y, Z);
  }
  char line[256];
  std::snprintf(line, sizeof(line), "DE = %f ED = %f PD = %f DIC = %f", dic[0], dic[1],
                dic[2], dic[3]);
  std::printf("%s\n", line);
  write_text("DIC.dat", std::string(line) + "\n");
  char sl[128];  // main.cu:430-432
  std::snprintf(sl, sizeof(sl), "%llu %llu %llu\n", (unsigned long long)seed[0],
                (unsigned long long)seed[1], (unsigned long long)seed[2]);
  write_text("seed.dat", sl);
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 7 && argc != 9) {
    std::printf("%s", kUsage);
    return 1;
  }
  char *e1 = nullptr, *e2 = nullptr, *e3 = nullptr;
  const long ntypes = std::strtol(argv[1], &e1, 10), ncov = std::strtol(argv[2], &e2, 10),
             gpu = std::strtol(argv[3], &e3, 10);
  if (*e1 || *e2 || *e3) {
    std::printf("%s", kUsage);
    return 1;
  }
  const std::string design = argv[4], mask_arg = argv[5], wm_arg = argv[6];
  int maxiter = 100000, burnin = 50000;
  if (argc == 9) {
    maxiter = std::atoi(argv[7]);
    burnin = std::atoi(argv[8]);
    if (maxiter < 1000)
      std::printf("WARNING: Silly-small number of iterations used; recommend abort and use "
                  "more\n");
    if (burnin > maxiter)
      std::printf("WARNING: Burn-in exceeds MAXITER, no results will be saved\n");
  }
  try {
    if (gpu != 1)
      throw InputError("GPU = 0 (the reference's untested CPU path) is not provided");
    if (ntypes < 0 || ncov < 1 || ncov > BSG_MAX_COVAR)
      throw InputError("NCov must be 1.." + std::to_string(BSG_MAX_COVAR));
    const std::string mask_name = mask_arg == "1" ? "mask.nii.gz" : mask_arg;
    const std::string wm_name =
        wm_arg == "0" ? "" : (wm_arg == "1" ? "avg152T1_white.nii.gz" : wm_arg);
    return run((int)ntypes, (int)ncov, design, mask_name, wm_name, maxiter, burnin);
  } catch (const InputError &e) {
    std::fprintf(stderr, "Error: %s\n", e.what());
    return 2;
  } catch (const SamplerError &e) {
    std::fprintf(stderr, "Error: %s\n", e.what());
    return 3;
  }
}
