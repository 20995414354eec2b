// bsg_internal.h -- device-side descriptors shared by the kernels and the
// host engine of libbsglmm_gb300.so.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace bsg {

constexpr int kMaxP = 8;                            // covariates per chain
constexpr int kMaxPairs = kMaxP * (kMaxP + 1) / 2;  // lower-triangle pairs
constexpr int kPostVals = kMaxPairs + kMaxP;        // pairs + column sums
// Partial rows of the colour kernels: colour 0 holds the column sums and the
// beta_WM term, colour 1 the pairs, the column sums and the beta_WM term.
constexpr int kP0Vals = kMaxP + 1;
constexpr int kFusedVals = kPostVals + 1;
constexpr int kWmOff = kPostVals;                    // beta_WM term's slot
constexpr int kChunk = 1024;                        // subjects staged per pass
constexpr int kChunkPad = kChunk + kChunk / 32;     // one pad word per 32
constexpr float kATail = 5.0f;  // inversion below, rejection above
constexpr int kTailMax = 16;    // rejection attempts per latent draw
constexpr int kGammaMax = 64;   // Marsaglia-Tsang attempts per gamma draw
constexpr int kPostThreads = 256;   // block shape of the allocation-free
constexpr int kPostPerThread = 4;   // Omega pass (bsg_noalloc.cu)
constexpr int kMaxThreads = 256;    // largest block of the colour kernel
constexpr int kPredThreads = 128;   // subjects per block of the predictive pass
constexpr int kPredWarps = 8;       // subjects (one warp each) per finishing block
constexpr int kF64Threads = 128;    // voxels (one thread each) per FP64-chain block

// Predictive-pass modes: after each kept sweep (ED and Qhat accumulate), on
// demand (Mpredict of the current coefficients), or the DE deviance at the
// posterior means.
enum : int { kPredKept = 0, kPredNow = 1, kPredDE = 2 };

// Philox counter tags: c3 = chain << 8 | tag.
enum : uint32_t {
  kTagZ = 1,
  kTagZTail = 2,
  kTagBeta = 3,
  kTagWNorm = 4,
  kTagGamma = 5,
  kTagWm = 6,
  kTagPhi = 7,      // scale-mixture weight draws (t/logit links)
  kTagPhiMore = 8,  // their further attempts
};

// Sticky per-chain error bits (ChainDev::status).
enum : int {
  kErrTnCap = 1,
  kErrChol = 2,
  kErrNaN = 4,
  kErrGammaCap = 8,
  kErrWishart = 16,
  kErrInput = 32,
};

// Read-only study data on the device.
struct DatasetDev {
  int32_t N, P, S, V, Vp, W;   // W = ceil(N / 32) outcome words per voxel
  int32_t n[2];                // voxels per colour
  const float *covar;          // [P][N]
  const float *xtx;            // [P][P]  X'X in float (read_data.cpp:321)
  const float *wm;             // [V] or nullptr (WM = 1)
  const float *xsum;           // [P] sum over subjects of each design column
  const float *cvec;           // [P] c with X c = 1 (all subjects), if has_c
  int32_t has_c;               // the design spans the constant
  double wm2;                  // sum over in-mask voxels of WM_v^2
  const int32_t *nb[2];        // [7][n_c]: sc(self), sc of the 6 neighbours
                               // in the order -x, +x, -y, +y, -z, +z
  const uint8_t *nbm[2];       // [n_c] bit t set iff neighbour t is in mask
  const int32_t *vidx[2];      // [n_c] compact mask index
  const uint32_t *ybits[2];    // [W][n_c] outcome bits, bit b = subject 32w+b
};

// Sampler state of one chain on the device.
struct ChainDev {
  int32_t dataset;
  uint32_t key0, key1, chain_id;
  float *wm_beta;          // [1] beta_WM, the white-matter coefficient
  double *wm_sum;          // [1] sum of beta_WM over kept sweeps
  int32_t wm_update;       // draw beta_WM | Z, beta every sweep
  // Link (the reference's MODEL, main.cu:42,168-175): 1 probit; 0 logistic
  // and 2 t, both as a t scale mixture of normals with weights phi.
  int32_t model;
  float t_df;              // nu of the t link (8 logistic, 3 t)
  float inv_lf;            // 1 / logit_factor (0.634 logistic, 1 t)
  float mix_d, mix_c;      // Marsaglia-Tsang d, c of Gamma((nu + 1) / 2)
  float *phi[2];           // [N][n_c] per colour: weights (t/logit links)
  int32_t df_offset, burnin, thin;
  float *beta;             // [P][Vp]
  // FP64 chain: the whole sweep in double precision on the same counters;
  // beta64 holds the coefficients and beta a float copy of them
  int32_t fp64;
  double *beta64;          // [P][Vp] (FP64 chains only)
  float *omega_f;          // [P*P] float copy read by the colour kernels
  double *omega_d;         // [P*P]
  float *colmean;          // [P]
  double *acc_sum;         // [P][V]  sum of beta over kept sweeps
  double *acc_sq;          // [P][V]  sum of beta^2
  double *prb_sum;         // [S][V]  sum of the lesion probability
  double *partials0;       // [kP0Vals][pstride0] column sums, WM term of
                           // each colour-0 block (value-major)
  double *partials1;       // [kFusedVals][pstride1] pairs, column sums, WM
                           // term of each colour-1 block (value-major)
  int32_t pstride0, pstride1;  // block rows allocated per value
  double *tot0;            // [kP0Vals] colour-0 totals of the sweep
  double *wdraw;           // [kMaxP + kMaxPairs] the sweep's Bartlett variates:
                           // sqrt(chi^2) diagonal, then the normals
  unsigned int *done;      // [2] arrival counters of the colour kernels
  long long *sweep;        // [2] sweeps completed by the colour-c kernel;
                           // sweep[1] is the chain's completed-sweep count
  long long *nkept;        // kept sweeps accumulated
  int *status;             // sticky error bits of this chain
  int *any_status;         // the context's OR of every chain's bits
  // DIC / Qhat predictive pass (null until first used)
  int32_t pred_tiles;      // voxel tiles of the predictive pass
  int32_t pred_tile;       // voxels per tile (a multiple of kPredThreads)
  double *pred_part;       // [N][max(S,1)][tiles] per-tile subject sums
  double *pred_subj;       // [N] each subject's term of the ED / DE sum
  double *mpred;           // [N][S] Mpredict of the last pass
  double *qhat;            // [N][S] Qhat, log scale (mcmc.cpp:223-225)
  double *pred_sums;       // [2] ED sum over kept sweeps; DE of the last DE pass
  long long *npred;        // kept sweeps the pass has seen
  unsigned int *pred_done; // arrival counter of the finishing kernel
};

// Parity mode: variates supplied by the caller instead of Philox.
struct Supplied {
  const uint32_t *ubits;   // [N][V]
  const float *normals;    // [V][P]
  const double *chi2;      // [P]
  const double *wnorm;     // [P(P-1)/2]
  int form;                // 0 reference draw, 1 production draw
};

struct BlockMap {
  int32_t chain;
  int32_t start;  // first colour position (fused) or merged position (post)
};

// ---- launchers (bsg_kernels.cu) ----------------------------------------
cudaError_t launch_fused(int P, int lpv, int threads, bool supplied,
                         const DatasetDev *ds, ChainDev *ch,
                         const BlockMap *map, int nblocks, int colour,
                         const Supplied &sup, cudaStream_t st,
                         bool pdl = false);
// The colour kernel of chains that draw beta_WM (one lane per voxel, Philox).
cudaError_t launch_fused_wm(int P, int threads, const DatasetDev *ds, ChainDev *ch,
                            const BlockMap *map, int nblocks, int colour,
                            cudaStream_t st, bool pdl);
// The colour kernel of the t/logit links (kMixLpv lanes per voxel, Philox).
constexpr int kMixLpv = 2;
cudaError_t launch_fused_mix(int P, int threads, const DatasetDev *ds, ChainDev *ch,
                             const BlockMap *map, int nblocks, int colour,
                             cudaStream_t st, bool pdl);
// The probit colour kernel with X'Z on the tensor cores (BF16x3 split, one
// lane per voxel, Philox), bsg_fused_tc.cu.
cudaError_t launch_fused_tc(int P, int threads, const DatasetDev *ds, ChainDev *ch,
                            const BlockMap *map, int nblocks, int colour, cudaStream_t st,
                            bool pdl);
// Its dynamic shared memory opt-in, before the first launch on a device.
cudaError_t prepare_fused_tc();
// The probit colour kernel (wmu: with the beta_WM update) on the 16-subject
// whole-word step, one lane per voxel, Philox (bsg_fused_wide.cu).
cudaError_t launch_fused_wide(int P, int threads, bool wmu, const DatasetDev *ds,
                              ChainDev *ch, const BlockMap *map, int nblocks, int colour,
                              cudaStream_t st, bool pdl);
// The colour kernel of FP64 chains (bsg_fp64.cu): one thread per voxel,
// kF64Threads voxels per block, Philox variates, probit link.
cudaError_t launch_fp64(int P, const DatasetDev *ds, ChainDev *ch, const BlockMap *map,
                        int nblocks, int colour, cudaStream_t st);
cudaError_t launch_prb(const DatasetDev *ds, const ChainDev *ch, int chain,
                       const DatasetDev &dh, float *prb, cudaStream_t st);
cudaError_t launch_fill(float *p, size_t n, float value, cudaStream_t st);
cudaError_t launch_pack(const uint8_t *bytes, int N, int V, int nc,
                        const int32_t *vidx, uint32_t *ybits, int *status,
                        cudaStream_t st);
bool fused_supported(int P, int lpv, int threads);
// Predictive pass (bsg_predict.cu).  With map == nullptr the grid is one
// chain's tiles (blockIdx.x) or subject blocks; otherwise map[blockIdx.x]
// holds {chain, tile} / {chain, subject block}.  chunks = subject blocks
// of kPredThreads (gridDim.y).
cudaError_t launch_predict(int P, int S, const DatasetDev *ds, ChainDev *ch,
                           const BlockMap *map, int nblocks, int chunks, int chain,
                           int mode, cudaStream_t st, bool pdl);
// Resident blocks per SM of predict_kernel<P, S>, for sizing its tiles.
int predict_blocks_per_sm(int P, int S);
cudaError_t launch_predict_finish(const DatasetDev *ds, ChainDev *ch,
                                  const BlockMap *map, int nblocks, int chain,
                                  int mode, cudaStream_t st, bool pdl);

}  // namespace bsg
