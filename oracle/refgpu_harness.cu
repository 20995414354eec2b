// refgpu_harness.cu -- TEST / MEASUREMENT INFRASTRUCTURE ONLY.
//
// Runs the reference's own GPU sweep (nicholst/BSGLMM bsglmm/covarGPU.cu)
// on this GPU, to time the form the GB300 sampler replaces.  The
// reference's device code is compiled from its source tree to PTX by the
// oracle recipe (`make -C oracle refgpu-ptx`, output oracle/_ref/covarGPU.ptx);
// this file is host code only: it loads that PTX with the runtime's library
// API (JIT for the current GPU), finds the reference's kernels by name and
// drives them as the reference's launchers do (mcmc.cpp:314-394 calling
// updateZGPU covarGPU.cu:1625-1669, updateSpatCoefGPU covarGPU.cu:535-584 and
// updateSpatCoefPrecGPU covarGPU.cu:1063-1112): two Z_GPU1 launches (96
// threads, P*96 floats of shared memory), the Omega and X'X uploads into the
// kernels' __constant__ arrays, two Spat_Coef_Probit launches (192
// threads), P column-mean reductions each with its own cudaMalloc, copy back
// and cudaFree, P(P+1) Spat_Coef_Prec launches each followed by a blocking
// copy, and the Wishart draw on the host.  The host Wishart here is this
// file's own FP64 Bartlett draw (chol -> invert -> chol of S + I, df =
// V + 19 as covarGPU.cu:1104), not the reference's randgen.cpp; it costs
// microseconds at P <= 8.  With rg_set_model(0 or 2) it runs the t/logit
// links instead: Z_GPU2 and Phi_GPU per colour, then the weighted
// Spat_Coef (the MODEL != 1 branches of the same launchers).
//
// Only bench.py's reference arm and tests load this library (through
// oracle.py); the product never does.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace {

struct RefGpu {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t k_setup = nullptr, k_z = nullptr, k_beta = nullptr, k_reduce = nullptr,
               k_prec = nullptr;
  // the t/logit links (MODEL 0 and 2): Z_GPU2, Phi_GPU and the weighted
  // Spat_Coef (covarGPU.cu:398-513,1430-1563)
  cudaKernel_t k_z2 = nullptr, k_phi = nullptr, k_beta_w = nullptr;
  int model = 1;
  float t_df = 1000.f;
  float *dphi = nullptr;
  void *d_prec_sym = nullptr, *d_xtx_sym = nullptr;
  // study
  int N = 0, P = 0, V = 0, Vp = 0, X = 0, Y = 0, n[2] = {0, 0};
  std::vector<float> xtx;
  // device buffers
  float *dZ = nullptr, *dcovar = nullptr, *dwm = nullptr, *dbeta = nullptr;
  unsigned char *ddata = nullptr, *dnbrs[2] = {nullptr, nullptr};
  int *dvox[2] = {nullptr, nullptr}, *didx = nullptr, *didxsc = nullptr;
  void *dstates = nullptr;
  std::vector<float> omega;  // [P][P], float as the reference keeps it
  std::mt19937_64 rng;
  std::string err;
};

RefGpu g;

int fail(const std::string &m) {
  g.err = m;
  return 1;
}

#define RG_CK(call)                                                              \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) return fail(std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
int upload(T **dst, const T *src, size_t n) {
  RG_CK(cudaMalloc((void **)dst, sizeof(T) * (n ? n : 1)));
  if (n) RG_CK(cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice));
  return 0;
}

// --- host FP64 Wishart: Omega ~ Wishart(df, (S + I)^-1), Bartlett ---------
bool chol(std::vector<double> &A, int n) {  // lower, A[c + r n]
  for (int k = 0; k < n; ++k) {
    double d = A[k + k * n];
    if (!(d > 0)) return false;
    d = std::sqrt(d);
    A[k + k * n] = d;
    for (int j = k + 1; j < n; ++j) A[k + j * n] /= d;
    for (int j = k + 1; j < n; ++j)
      for (int i = j; i < n; ++i) A[j + i * n] -= A[k + i * n] * A[k + j * n];
  }
  return true;
}

void chol_inverse(const std::vector<double> &G, int n, std::vector<double> &out) {
  std::vector<double> col(n);
  for (int k = 0; k < n; ++k) {
    for (int i = 0; i < n; ++i) col[i] = (i == k) ? 1.0 : 0.0;
    for (int i = 0; i < n; ++i) {
      double s = col[i];
      for (int j = 0; j < i; ++j) s -= G[j + i * n] * col[j];
      col[i] = s / G[i + i * n];
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = col[i];
      for (int j = i + 1; j < n; ++j) s -= G[i + j * n] * col[j];
      col[i] = s / G[i + i * n];
    }
    for (int i = 0; i < n; ++i) out[k + i * n] = col[i];
  }
}

bool host_wishart(const std::vector<double> &S, double df) {
  const int P = g.P;
  std::vector<double> A(S), Ai(P * P), T(P * P, 0.0), B(P * P, 0.0);
  for (int i = 0; i < P; ++i) A[i + i * P] += 1.0;
  if (!chol(A, P)) return false;
  chol_inverse(A, P, Ai);
  if (!chol(Ai, P)) return false;
  std::normal_distribution<double> nd(0.0, 1.0);
  for (int i = 0; i < P; ++i) {
    std::chi_squared_distribution<double> cs(df - i);
    T[i + i * P] = std::sqrt(cs(g.rng));
    for (int j = 0; j < i; ++j) T[j + i * P] = nd(g.rng);
  }
  for (int i = 0; i < P; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = 0;
      for (int k = j; k <= i; ++k) s += Ai[k + i * P] * T[j + k * P];
      B[j + i * P] = s;
    }
  for (int i = 0; i < P; ++i)
    for (int j = 0; j < P; ++j) {
      const int K = i < j ? i : j;
      double s = 0;
      for (int k = 0; k <= K; ++k) s += B[k + i * P] * B[k + j * P];
      g.omega[j + i * P] = (float)s;
    }
  return true;
}

// --- one sweep in the reference's order ------------------------------------
int sweep() {
  const int P = g.P, nrow = g.X, ncol = g.Y, ncovfix = 0, nsubtypes = 1;
  const float beta_wm = 0.f, sqrt2 = std::sqrt(2.f);
  void *nullp = nullptr;
  // updateZGPU (covarGPU.cu:1625-1669): Z_GPU2 (t/logit links) or Z_GPU1
  // per colour; then updatePhiGPU (covarGPU.cu:1590-1612): Phi_GPU
  if (g.model != 1) {
    const float alp = (g.t_df + 1.f) / 2.f, df = g.t_df;
    for (int pass = 0; pass < 2; ++pass)
      for (int c = 0; c < 2; ++c) {
        const int tpb = 96, nb = (g.n[c] + tpb - 1) / tpb;
        if (nb == 0) continue;
        int N = g.N, NC = g.n[c], Vp = g.Vp, V = g.V;
        void *a_z[] = {&g.dZ,  &g.ddata, &g.dcovar, &nullp,  &nullp, &nullp, &g.dwm,
                       &g.dbeta, (void *)&beta_wm, &g.dvox[c], &N, (void *)&nsubtypes,
                       (void *)&P, (void *)&ncovfix, &NC, &Vp, &V, &g.dstates, &g.didx,
                       &g.didxsc, (void *)&sqrt2, &g.dphi, &nullp, (void *)&alp,
                       (void *)&df};
        void *a_phi[] = {&g.dZ,  &g.ddata, &g.dcovar, &nullp,  &nullp, &nullp, &g.dwm,
                         &g.dbeta, (void *)&beta_wm, &g.dvox[c], &N, (void *)&nsubtypes,
                         (void *)&P, (void *)&ncovfix, &NC, &Vp, &V, &g.dstates, &g.didx,
                         &g.didxsc, (void *)&sqrt2, &g.dphi, (void *)&alp, (void *)&df};
        RG_CK(cudaLaunchKernel((const void *)(pass == 0 ? g.k_z2 : g.k_phi), dim3(nb),
                               dim3(tpb), pass == 0 ? a_z : a_phi, sizeof(float) * P * tpb,
                               0));
      }
  }
  for (int c = 0; c < 2 && g.model == 1; ++c) {
    const int tpb = 96, nb = (g.n[c] + tpb - 1) / tpb;
    if (nb == 0) continue;
    int N = g.N, NC = g.n[c], Vp = g.Vp, V = g.V;
    void *args[] = {&g.dZ,   &g.ddata, &g.dcovar, &nullp,  &nullp,  &nullp,      &g.dwm,
                    &g.dbeta, (void *)&beta_wm,   &g.dvox[c], &N,    (void *)&nsubtypes,
                    (void *)&P, (void *)&ncovfix, &NC, &Vp, &V, &g.dstates, &g.didx,
                    &g.didxsc, (void *)&sqrt2, &nullp};
    RG_CK(cudaLaunchKernel((const void *)g.k_z, dim3(nb), dim3(tpb), args,
                           sizeof(float) * P * tpb, 0));
  }
  // updateSpatCoefGPU (covarGPU.cu:535-584)
  RG_CK(cudaMemcpy(g.d_prec_sym, g.omega.data(), sizeof(float) * P * P,
                   cudaMemcpyHostToDevice));
  RG_CK(cudaMemcpy(g.d_xtx_sym, g.xtx.data(), sizeof(float) * P * P,
                   cudaMemcpyHostToDevice));
  for (int c = 0; c < 2; ++c) {
    const int tpb = 192, nb = (g.n[c] + tpb - 1) / tpb;
    if (nb == 0) continue;
    int N = g.N, NC = g.n[c], Vp = g.Vp, V = g.V, X = nrow, Y = ncol;
    void *args[] = {&g.dcovar, &nullp,  &nullp,  &nullp,    &g.dZ,   &g.dwm,
                    &g.dbeta,  (void *)&beta_wm, &g.dnbrs[c], &g.dvox[c], &N, &X, &Y,
                    (void *)&nsubtypes, (void *)&P, (void *)&ncovfix, &NC, &Vp, &V,
                    &g.dstates, &g.didx, &g.didxsc};
    // the weighted update takes Phi after Z (covarGPU.cu:398)
    void *args_w[] = {&g.dcovar, &nullp,  &nullp,  &nullp,    &g.dZ,   &g.dphi, &g.dwm,
                      &g.dbeta,  (void *)&beta_wm, &g.dnbrs[c], &g.dvox[c], &N, &X, &Y,
                      (void *)&nsubtypes, (void *)&P, (void *)&ncovfix, &NC, &Vp, &V,
                      &g.dstates, &g.didx, &g.didxsc};
    RG_CK(cudaLaunchKernel((const void *)(g.model == 1 ? g.k_beta : g.k_beta_w), dim3(nb),
                           dim3(tpb), g.model == 1 ? args : args_w, sizeof(float) * P * tpb,
                           0));
  }
  const int BPG = 32;
  for (int p = 0; p < P; ++p) {  // column means, one allocation each
    float *dsum = nullptr;
    RG_CK(cudaMalloc((void **)&dsum, BPG * sizeof(float)));
    float *in = g.dbeta + (size_t)p * g.Vp;
    int Vp = g.Vp;
    void *args[] = {&in, &dsum, &Vp};
    RG_CK(cudaLaunchKernel((const void *)g.k_reduce, dim3(BPG), dim3(256), args, 0, 0));
    float h[32];
    RG_CK(cudaMemcpy(h, dsum, sizeof(h), cudaMemcpyDeviceToHost));
    RG_CK(cudaFree(dsum));
  }
  // updateSpatCoefPrecGPU (covarGPU.cu:1063-1112)
  float *dpart = nullptr;
  RG_CK(cudaMalloc((void **)&dpart, BPG * sizeof(float)));
  RG_CK(cudaMemset(dpart, 0, BPG * sizeof(float)));
  std::vector<double> S((size_t)P * P, 0.0);
  for (int ii = 0; ii < P; ++ii)
    for (int jj = 0; jj <= ii; ++jj) {
      for (int c = 0; c < 2; ++c) {
        float *b1 = g.dbeta + (size_t)ii * g.Vp, *b2 = g.dbeta + (size_t)jj * g.Vp;
        int NC = g.n[c], X = nrow, Y = ncol;
        void *args[] = {&b1, &b2, &NC, &X, &Y, &g.dvox[c], &dpart, &g.didxsc};
        RG_CK(cudaLaunchKernel((const void *)g.k_prec, dim3(BPG), dim3(256), args, 0, 0));
        float h[32];
        RG_CK(cudaMemcpy(h, dpart, sizeof(h), cudaMemcpyDeviceToHost));
        for (int j = 0; j < BPG; ++j) S[jj + ii * P] += (double)h[j];
      }
      S[ii + jj * P] = S[jj + ii * P];
    }
  RG_CK(cudaFree(dpart));
  if (!host_wishart(S, (double)g.V + 19.0)) return fail("host Wishart: S + I not SPD");
  return 0;
}

}  // namespace

extern "C" {

const char *rg_error() { return g.err.c_str(); }

// Loads the reference's PTX and finds its kernels.  Returns 0 on success.
int rg_open(const char *ptx_path, int device) {
  RG_CK(cudaSetDevice(device));
  FILE *f = std::fopen(ptx_path, "rb");
  if (!f) return fail(std::string("cannot open ") + ptx_path);
  std::vector<char> text;
  char buf[1 << 16];
  size_t r;
  while ((r = std::fread(buf, 1, sizeof(buf), f)) > 0) text.insert(text.end(), buf, buf + r);
  std::fclose(f);
  text.push_back('\0');
  RG_CK(cudaLibraryLoadData(&g.lib, text.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
  unsigned int nk = 0;
  RG_CK(cudaLibraryGetKernelCount(&nk, g.lib));
  std::vector<cudaKernel_t> ks(nk);
  RG_CK(cudaLibraryEnumerateKernels(ks.data(), nk, g.lib));
  // the kernels by their length-prefixed (mangled) names
  const struct {
    const char *tag;
    cudaKernel_t *dst;
  } want[] = {{"12setup_kernel", &g.k_setup},
              {"6Z_GPU1", &g.k_z},
              {"16Spat_Coef_Probit", &g.k_beta},
              {"6reduce", &g.k_reduce},
              {"14Spat_Coef_Prec", &g.k_prec},
              {"6Z_GPU2", &g.k_z2},
              {"7Phi_GPU", &g.k_phi},
              {"9Spat_Coef", &g.k_beta_w}};
  std::string names;
  for (cudaKernel_t k : ks) {
    const char *name = nullptr;
    if (cudaFuncGetName(&name, (const void *)k) != cudaSuccess || !name) continue;
    names += std::string(name) + " ";
    for (const auto &w : want)
      if (std::strncmp(name, "_Z", 2) == 0 && std::strstr(name, w.tag) == name + 2)
        *w.dst = k;
  }
  for (const auto &w : want)
    if (!*w.dst) return fail(std::string("kernel not found: ") + w.tag + " among " + names);
  size_t sz = 0;
  RG_CK(cudaLibraryGetGlobal(&g.d_prec_sym, &sz, g.lib, "dPrec"));
  RG_CK(cudaLibraryGetGlobal(&g.d_xtx_sym, &sz, g.lib, "dtmpvar"));
  return 0;
}

// The study in the reference's layouts: padded grid (X+2)(Y+2)(Z+2) maps
// idx / idxsc, per-colour voxel lists (padded indices) and in-mask
// neighbour counts, covar [P][N], data [N][V] bytes, X'X [P][P].
int rg_setup(int X, int Y, int Z, int N, int P, int V, int Vp, const int32_t *idx,
             const int32_t *idxsc, int n0, const int32_t *vox0, const uint8_t *nbrs0,
             int n1, const int32_t *vox1, const uint8_t *nbrs1, const float *covar,
             const uint8_t *data, const float *xtx, uint64_t seed) {
  if (N > 2000) return fail("the reference's Z_GPU1 holds at most 2000 subjects");
  if (P < 1 || P > 20) return fail("P out of the reference's range");
  g.X = X;
  g.Y = Y;
  g.N = N;
  g.P = P;
  g.V = V;
  g.Vp = Vp;
  g.n[0] = n0;
  g.n[1] = n1;
  g.xtx.assign(xtx, xtx + P * P);
  g.omega.assign((size_t)P * P, 0.f);
  for (int i = 0; i < P; ++i) g.omega[i + i * P] = 1.f;  // mcmc.cpp:149-154
  g.rng.seed(seed);
  const size_t nsize = (size_t)(X + 2) * (Y + 2) * (Z + 2);
  if (upload(&g.didx, idx, nsize) || upload(&g.didxsc, idxsc, nsize) ||
      upload(&g.dvox[0], vox0, (size_t)n0) || upload(&g.dvox[1], vox1, (size_t)n1) ||
      upload(&g.dnbrs[0], nbrs0, (size_t)n0) || upload(&g.dnbrs[1], nbrs1, (size_t)n1) ||
      upload(&g.dcovar, covar, (size_t)P * N) || upload(&g.ddata, data, (size_t)N * V))
    return 1;
  std::vector<float> wm((size_t)V, 1.f);  // WM argument 0: WM = 1 (read_data.cpp:534)
  if (upload(&g.dwm, wm.data(), wm.size())) return 1;
  RG_CK(cudaMalloc((void **)&g.dZ, sizeof(float) * (size_t)N * V));
  RG_CK(cudaMemset(g.dZ, 0, sizeof(float) * (size_t)N * V));
  RG_CK(cudaMalloc((void **)&g.dbeta, sizeof(float) * (size_t)P * Vp));
  RG_CK(cudaMemset(g.dbeta, 0, sizeof(float) * (size_t)P * Vp));
  // one XORWOW state per slot of the larger colour (main.cu:396-415); a
  // curandStateXORWOW is 48 bytes
  const int nmax = n0 > n1 ? n0 : n1;
  RG_CK(cudaMalloc(&g.dstates, (size_t)48 * (nmax ? nmax : 1)));
  unsigned long long dseed = (unsigned long long)seed;
  int nst = nmax;
  void *args[] = {&g.dstates, &dseed, &nst};
  RG_CK(cudaLaunchKernel((const void *)g.k_setup, dim3(512), dim3(512), args, 0, 0));
  RG_CK(cudaDeviceSynchronize());
  return 0;
}

// The link, the reference's compile-time MODEL (main.cu:42,168-175): 1
// probit; 0 logistic (t_8 mixture) and 2 t (t_3), with the scale-mixture
// weights Phi (N V floats) allocated here and set to 1, the value of the
// reference's restart code (mcmc.cpp:1245): its own allocation of devicePhi
// is commented out (mcmc.cpp:179-180), so this path cannot run as shipped.
// The weighted Spat_Coef stages the design only from threads with a voxel,
// so every colour must fill whole 192-voxel blocks (the caller's study
// guarantees it; rg_set_model refuses otherwise).
int rg_set_model(int model) {
  if (model < 0 || model > 2) return fail("model must be 0, 1 or 2");
  if (model != 1 && (g.n[0] % 192 || g.n[1] % 192))
    return fail("the t/logit kernels need colour sizes that are multiples of 192");
  g.model = model;
  g.t_df = model == 0 ? 8.f : (model == 2 ? 3.f : 1000.f);
  if (model != 1 && !g.dphi) {
    const size_t n = (size_t)g.N * g.V;
    std::vector<float> ones(n, 1.f);
    if (upload(&g.dphi, ones.data(), n)) return 1;
  }
  return 0;
}

// Runs n sweeps; *ms = host wall time per sweep (the reference's loop is
// host-synchronous: every launcher ends in a blocking copy).
int rg_sweeps(int n, double *ms) {
  cudaEvent_t a, b;
  RG_CK(cudaEventCreate(&a));
  RG_CK(cudaEventCreate(&b));
  RG_CK(cudaDeviceSynchronize());
  RG_CK(cudaEventRecord(a, 0));
  for (int i = 0; i < n; ++i)
    if (sweep()) return 1;
  RG_CK(cudaEventRecord(b, 0));
  RG_CK(cudaEventSynchronize(b));
  float t = 0;
  RG_CK(cudaEventElapsedTime(&t, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (ms) *ms = (double)t / (n > 0 ? n : 1);
  return 0;
}

int rg_get_beta(float *out) {
  RG_CK(cudaMemcpy(out, g.dbeta, sizeof(float) * (size_t)g.P * g.Vp, cudaMemcpyDeviceToHost));
  return 0;
}

int rg_get_omega(float *out) {
  std::memcpy(out, g.omega.data(), sizeof(float) * g.omega.size());
  return 0;
}

void rg_close() {
  cudaFree(g.dZ);
  cudaFree(g.dcovar);
  cudaFree(g.dwm);
  cudaFree(g.dbeta);
  cudaFree(g.ddata);
  for (int c = 0; c < 2; ++c) {
    cudaFree(g.dnbrs[c]);
    cudaFree(g.dvox[c]);
  }
  cudaFree(g.didx);
  cudaFree(g.didxsc);
  cudaFree(g.dphi);
  cudaFree(g.dstates);
  if (g.lib) cudaLibraryUnload(g.lib);
  g = RefGpu();
}

}  // extern "C"
