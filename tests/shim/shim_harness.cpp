// shim_harness.cpp -- test driver of covarGPU_shim.cu.  It plays the part of
// the reference's main.cu / mcmc.cpp: defines their globals, fills them from
// a study file and calls the launchers in the order of mcmc.cpp's GPU branch
// (mcmc.cpp:318,356,367,595,605-607) for a number of sweeps, keeping every
// sweep after the first, then writes the resulting Omega, coefficients,
// lesion probabilities, the ED sum and Qhat.
//
// usage: shim_harness <study.bin> <sweeps> <out.bin> [wm | model=M]
// With "wm" the study file also holds V floats of WM after the seed and the
// harness calls updateBetaGPU before each coefficient update (UPDATE_WM);
// with "model=M" MODEL is M and updatePhiGPU follows updateZGPU
// (mcmc.cpp:327-329).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

// ---- the reference's globals --------------------------------------------
int NSUBS, NROW, NCOL, NDEPTH, TOTVOX, TOTVOXp, NCOVAR, NSUBTYPES;
int UPDATE_WM = 0, MODEL = 1;
float logit_factor = 1.0f;
int *hostIdx = nullptr;
float *deviceSpatCoef = nullptr;
float *devicePrb = nullptr;

// KISS with 64-bit words and the 2^-64 scale of PREC = 64, as the
// reference's randgen.cpp:9-23 (provided by randgen.cpp in a real build).
double kiss(unsigned long *s) {
  s[1] = s[1] ^ (s[1] << 17);
  s[2] = (s[2] ^ (s[2] << 18)) & 0x7FFFFFFFul;
  s[0] = 69069ul * s[0] + 23606797ul;
  s[1] ^= (s[1] >> 15);
  s[2] ^= (s[2] >> 13);
  return (double)(s[0] + s[1] + s[2]) * 5.421010862427522e-20;
}

// ---- the launchers the shim defines (mcmc.cpp:101-125) ----------------
void updateZGPU(unsigned char *, float, unsigned long *);
void updateSpatCoefGPU(float *, float *, float *, float *, float *, float *,
                       float *, unsigned char *, float, float *, unsigned long *);
void updateSpatCoefPrecGPU(float *, unsigned long *);
void updatePhiGPU(float, float *);
void updateBetaGPU(float *, float *, float *, float *, float *, float, float,
                   float *, float *, unsigned long *);
void compute_prbGPU(float);
double compute_predictGPU(float, unsigned char *, unsigned char *, float *,
                          float *, double **, int);

template <typename T>
std::vector<T> rd(FILE *f, size_t n) {
  std::vector<T> v(n);
  if (n && fread(v.data(), sizeof(T), n, f) != n) {
    std::fprintf(stderr, "short read\n");
    std::exit(2);
  }
  return v;
}

int main(int argc, char **argv) {
  if (argc != 4 && argc != 5) return 2;
  UPDATE_WM = argc == 5 && std::string(argv[4]) == "wm";
  if (argc == 5 && std::string(argv[4]).rfind("model=", 0) == 0)
    MODEL = std::atoi(argv[4] + 6);
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  auto hdr = rd<int32_t>(f, 8);
  NROW = hdr[0], NCOL = hdr[1], NDEPTH = hdr[2], NSUBS = hdr[3];
  NCOVAR = hdr[4], NSUBTYPES = hdr[5], TOTVOX = hdr[6], TOTVOXp = hdr[7];
  const size_t nsize = (size_t)(NROW + 2) * (NCOL + 2) * (NDEPTH + 2);
  auto idx = rd<int32_t>(f, nsize);
  auto covar = rd<float>(f, (size_t)NCOVAR * NSUBS);
  auto data = rd<uint8_t>(f, (size_t)NSUBS * TOTVOX);
  auto seed0 = rd<uint64_t>(f, 3);
  std::vector<float> wm(TOTVOX, 1.0f);
  if (UPDATE_WM) wm = rd<float>(f, TOTVOX);
  std::fclose(f);
  hostIdx = idx.data();
  unsigned long seed[3] = {(unsigned long)seed0[0], (unsigned long)seed0[1],
                           (unsigned long)seed0[2]};
  cudaMalloc(&deviceSpatCoef, sizeof(float) * (size_t)NCOVAR * TOTVOXp);
  cudaMalloc(&devicePrb, sizeof(float) * ((size_t)NSUBTYPES * TOTVOX + 1));
  // mcmc.cpp:149-154: Omega = I
  std::vector<float> prec((size_t)NCOVAR * NCOVAR, 0.f), mean(NCOVAR, 0.f);
  std::vector<float> alphaMean(NCOVAR, 0.f);
  for (int i = 0; i < NCOVAR; ++i) prec[i + i * NCOVAR] = 1.f;
  std::vector<float> spatCoef((size_t)NCOVAR * TOTVOXp, 0.f);
  const int sweeps = std::atoi(argv[2]);
  float beta = 0.f;
  std::vector<double> qstore((size_t)NSUBS * (NSUBTYPES > 0 ? NSUBTYPES : 1), 0.0);
  std::vector<double *> Qhat(NSUBS);  // mcmc.cpp:223-225
  for (int i = 0; i < NSUBS; ++i) Qhat[i] = &qstore[(size_t)i * NSUBTYPES];
  double ED = 0.0;
  int totsav = 0;
  for (int iter = 0; iter < sweeps; ++iter) {
    updateZGPU(data.data(), beta, seed);
    if (MODEL != 1) updatePhiGPU(beta, nullptr);  // mcmc.cpp:327-329
    if (UPDATE_WM)  // mcmc.cpp:344-345
      updateBetaGPU(&beta, nullptr, nullptr, nullptr, nullptr, 0.f, 1e-6f, nullptr,
                    nullptr, seed);
    updateSpatCoefGPU(covar.data(), spatCoef.data(), mean.data(), prec.data(),
                      nullptr, alphaMean.data(), nullptr, nullptr, beta,
                      wm.data(), seed);
    updateSpatCoefPrecGPU(prec.data(), seed);
    if (iter > 0) {  // BURNIN = 0, SAVE_ITER = 1
      ED += compute_predictGPU(beta, data.data(), nullptr, covar.data(), nullptr,
                               Qhat.data(), totsav == 0);
      ++totsav;
    }
  }
  if (UPDATE_WM)  // the beta_WM the next iteration would start from
    updateBetaGPU(&beta, nullptr, nullptr, nullptr, nullptr, 0.f, 1e-6f, nullptr,
                  nullptr, seed);
  compute_prbGPU(beta);
  std::vector<float> prb((size_t)NSUBTYPES * TOTVOX);
  cudaMemcpy(spatCoef.data(), deviceSpatCoef, sizeof(float) * spatCoef.size(),
             cudaMemcpyDeviceToHost);
  cudaMemcpy(prb.data(), devicePrb, sizeof(float) * prb.size(), cudaMemcpyDeviceToHost);
  FILE *o = std::fopen(argv[3], "wb");
  fwrite(prec.data(), sizeof(float), prec.size(), o);
  fwrite(spatCoef.data(), sizeof(float), spatCoef.size(), o);
  fwrite(prb.data(), sizeof(float), prb.size(), o);
  fwrite(alphaMean.data(), sizeof(float), alphaMean.size(), o);
  unsigned long long s3[3] = {seed[0], seed[1], seed[2]};
  fwrite(s3, 8, 3, o);
  fwrite(&ED, sizeof(double), 1, o);
  fwrite(qstore.data(), sizeof(double), qstore.size(), o);
  fwrite(&beta, sizeof(float), 1, o);
  std::fclose(o);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
