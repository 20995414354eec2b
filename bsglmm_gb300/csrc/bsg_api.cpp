// bsg_api.cpp -- host engine behind the C ABI of bsglmm_gb300.h: lattice
// construction, uploads, chain state, the per-sweep launch plan, CUDA-graph
// segments, status reporting and read-back.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/bsglmm_gb300.h"
#include "bsg_internal.h"

using namespace bsg;

namespace {

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

struct Dataset {
  int X = 0, Y = 0, Z = 0, PX = 0, PY = 0, nsize = 0;
  int N = 0, P = 0, S = 0, V = 0, Vp = 0;
  std::vector<int32_t> idx, idxsc, vox[2];
  std::vector<uint8_t> nbrs[2];
  std::vector<int32_t> pad_of_v;  // padded index of compact mask index v
  DatasetDev dev{};               // device pointers
};

struct Chain {
  int dataset = 0;
  bsg_chain_desc desc{};
  ChainDev dev{};
  size_t cap0 = 0, cap1 = 0;  // partial rows allocated per colour
  bool pred_on = false;        // predictive pass after every kept sweep
};

struct Group {
  int P = 0;
  bool mix = false;     // t/logit chains (scale-mixture colour kernel)
  bool wm_any = false;  // its chains draw beta_WM: colour 0 waits for it
  bool fp64 = false;    // FP64 chains (fp64_colour_kernel, no early start)
  bool wide = false;    // the 16-subject whole-word step (bsg_fused_wide.cu)
  double vox = 0, subj_vox = 0;  // its chains' voxels and N x voxels
  std::vector<BlockMap> map[2];
  BlockMap *d_map[2] = {nullptr, nullptr};
  // predictive pass of the group's chains that have it on, one launch pair
  // per number of group columns S: {chain, tile} blocks, {chain, subject
  // block} finishing blocks, subject chunks
  struct Pred {
    int S = 0;
    std::vector<BlockMap> pmap, fmap;
    BlockMap *d_pmap = nullptr, *d_fmap = nullptr;
    int pchunks = 0;
  };
  std::vector<Pred> pred;
};

// beta_WM of one chain on the device.
struct WmState {
  double sum;   // over kept sweeps
  float beta;   // current value
  int pad;
};

// Small per-chain counters of the predictive pass.
struct PredCounters {
  long long npred;
  unsigned int done;
  int pad;
};

// Small per-chain counters kept together on the device.
struct ChainCounters {
  long long sweep[2];  // sweeps completed by the colour-0 / colour-1 kernel
  long long nkept;
  unsigned int done[2];
  int status;
};

}  // namespace

struct bsg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> join;
  cudaEvent_t fork = nullptr;
  std::vector<Dataset> ds;
  std::vector<Chain> ch;
  std::vector<DevBuf> owned;
  DatasetDev *d_ds = nullptr;
  ChainDev *d_ch = nullptr;
  size_t d_ds_cap = 0, d_ch_cap = 0;
  bool plan_valid = false;
  std::vector<Group> groups;
  int *any_status = nullptr;  // device word: OR of every chain's error bits
  int lpv = 1, threads = 256;
  bool tc = false;  // probit X'Z on the tensor cores (BF16x3 split)
  int step = 0;     // subjects per whole-word step: 8, 16, 0 = chosen per group
#ifdef BSG_NO_PDL
  bool pdl = false;
#else
  bool pdl = true;  // overlap each colour kernel's latent phase with the
                    // previous kernel's tail (programmatic dependent launch)
#endif
  std::map<int64_t, cudaGraphExec_t> graphs;
  void *pin = nullptr;  // pinned staging of bsg_step_host
  size_t pin_bytes = 0;
  bool pin_busy = false;  // copies through it may be in flight (a call ended early)
  std::string err;
};

namespace {

bsg_status fail(bsg_ctx *c, bsg_status s, const std::string &m) {
  if (c) c->err = m;
  return s;
}

#define CK(call)                                                           \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess)                                                 \
      return fail(ctx, BSG_ERR_CUDA,                                       \
                  std::string(#call) + ": " + cudaGetErrorString(e_));     \
  } while (0)

void *dalloc(bsg_ctx *ctx, size_t bytes, cudaError_t *e) {
  void *p = nullptr;
  *e = cudaMalloc(&p, bytes ? bytes : 4);
  if (*e != cudaSuccess) return nullptr;
  ctx->owned.push_back({p, bytes});
  return p;
}

// Every copy and fill runs on the context stream, so that it is ordered with
// the sweep kernels (the context stream is non-blocking: work on the legacy
// default stream would race it).  A pageable host source is staged before
// cudaMemcpyAsync returns; a page-locked one is read later by the copy
// engine, so the copy is waited for before the caller may reuse the buffer.
// A device-to-host copy is always waited for.
cudaError_t h2d(bsg_ctx *ctx, void *dst, const void *src, size_t n) {
  cudaError_t e = cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) return e;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, src) != cudaSuccess) {
    cudaGetLastError();
    return cudaStreamSynchronize(ctx->stream);
  }
  return a.type == cudaMemoryTypeUnregistered ? cudaSuccess
                                              : cudaStreamSynchronize(ctx->stream);
}

cudaError_t d2h(bsg_ctx *ctx, void *dst, const void *src, size_t n) {
  cudaError_t e = cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, ctx->stream);
  return e != cudaSuccess ? e : cudaStreamSynchronize(ctx->stream);
}

void dfree(bsg_ctx *ctx, void *p) {
  if (!p) return;
  for (size_t i = 0; i < ctx->owned.size(); ++i)
    if (ctx->owned[i].p == p) {
      cudaFree(p);
      ctx->owned.erase(ctx->owned.begin() + i);
      return;
    }
}

void clear_graphs(bsg_ctx *ctx) {
  for (auto &kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
  ctx->graphs.clear();
}

// Lattice of main.cu: padding by one voxel (main.cu:56), 6-neighbour
// dilation (main.cu:189-205), compact maps in padded scan order
// (main.cu:308-329), colour lists in interior scan order with colour 0 for
// i+j+k odd in 1-based padded coordinates (main.cu:216-252,333-394) and
// in-mask neighbour counts (cnt_nbrs, main.cu:471-502).
void build_lattice(Dataset &d, const uint8_t *mask) {
  const int X = d.X, Y = d.Y, Z = d.Z;
  d.PX = X + 2;
  d.PY = Y + 2;
  const int PZ = Z + 2, sy = d.PX, sz = d.PX * d.PY;
  d.nsize = d.PX * d.PY * PZ;
  std::vector<uint8_t> msk(d.nsize, 0), mskp(d.nsize, 0);
  size_t t = 0;
  for (int k = 1; k <= Z; ++k)
    for (int j = 1; j <= Y; ++j)
      for (int i = 1; i <= X; ++i, ++t) msk[i + sy * j + sz * k] = mask[t] ? 1 : 0;
  for (int k = 1; k <= Z; ++k)
    for (int j = 1; j <= Y; ++j)
      for (int i = 1; i <= X; ++i) {
        const int p = i + sy * j + sz * k;
        if (!msk[p]) continue;
        mskp[p] = mskp[p - 1] = mskp[p + 1] = 1;
        mskp[p - sy] = mskp[p + sy] = mskp[p - sz] = mskp[p + sz] = 1;
      }
  d.idx.assign(d.nsize, -1);
  d.idxsc.assign(d.nsize, -1);
  int cnt = 0, cntp = 0;
  for (int p = 0; p < d.nsize; ++p) {
    if (msk[p]) d.idx[p] = cnt++;
    if (mskp[p]) d.idxsc[p] = cntp++;
  }
  d.V = cnt;
  d.Vp = cntp;
  d.pad_of_v.assign(d.V, 0);
  for (int c = 0; c < 2; ++c) {
    d.vox[c].clear();
    d.nbrs[c].clear();
  }
  for (int k = 1; k <= Z; ++k)
    for (int j = 1; j <= Y; ++j)
      for (int i = 1; i <= X; ++i) {
        const int p = i + sy * j + sz * k;
        if (!msk[p]) continue;
        d.pad_of_v[d.idx[p]] = p;
        const int c = ((i + j + k) & 1) ? 0 : 1;
        d.vox[c].push_back(p);
        d.nbrs[c].push_back((uint8_t)(msk[p - 1] + msk[p + 1] + msk[p - sy] +
                                      msk[p + sy] + msk[p - sz] + msk[p + sz]));
      }
}

template <typename T>
T *upload(bsg_ctx *ctx, const T *host, size_t n, cudaError_t *e) {
  T *p = (T *)dalloc(ctx, sizeof(T) * n, e);
  if (!p) return nullptr;
  if (n) *e = h2d(ctx, p, host, sizeof(T) * n);
  return *e == cudaSuccess ? p : nullptr;
}

bsg_status status_from_bits(int bits) {
  if (!bits) return BSG_OK;
  if (bits & kErrInput) return BSG_ERR_INVALID;
  if (bits & kErrNaN) return BSG_ERR_NAN;
  if (bits & (kErrChol | kErrWishart)) return BSG_ERR_NOT_SPD;
  if (bits & (kErrTnCap | kErrGammaCap)) return BSG_ERR_SAMPLER_CAP;
  return BSG_ERR_STATE;
}

std::string status_text(int bits) {
  std::string s;
  if (bits & kErrTnCap) s += " truncated-normal tail cap hit;";
  if (bits & kErrGammaCap) s += " gamma cap hit;";
  if (bits & kErrChol) s += " conditional precision of a voxel not SPD;";
  if (bits & kErrWishart) s += " Wishart scale not SPD;";
  if (bits & kErrNaN) s += " non-finite state;";
  if (bits & kErrInput) s += " outcome values outside {0,1};";
  return s;
}

constexpr int kParityThreads = 128;  // tile of the supplied-variate sweep

// Partials of the colour kernels, one per block of a chain and value
// (value-major, so that the last block's sums read consecutive blocks):
// column sums (colour 0) and pairs + column sums (colour 1), sized for the
// smallest tile the context launches; tot0 takes colour 0's totals.
bsg_status ensure_partials(bsg_ctx *ctx, int vpb) {
  cudaError_t e;
  for (auto &c : ctx->ch) {
    const Dataset &d = ctx->ds[c.dataset];
    const size_t n0 = std::max<size_t>(1, (d.vox[0].size() + vpb - 1) / vpb);
    const size_t n1 = std::max<size_t>(1, (d.vox[1].size() + vpb - 1) / vpb);
    if (n0 > c.cap0) {
      dfree(ctx, c.dev.partials0);
      c.dev.partials0 = (double *)dalloc(ctx, sizeof(double) * n0 * kP0Vals, &e);
      CK(e);
      c.cap0 = n0;
    }
    if (n1 > c.cap1) {
      dfree(ctx, c.dev.partials1);
      c.dev.partials1 = (double *)dalloc(ctx, sizeof(double) * n1 * kFusedVals, &e);
      CK(e);
      c.cap1 = n1;
    }
    if (!c.dev.tot0) {
      const size_t n = kP0Vals + kMaxP + kMaxPairs;
      c.dev.tot0 = (double *)dalloc(ctx, sizeof(double) * n, &e);
      CK(e);
      CK(cudaMemsetAsync(c.dev.tot0, 0, sizeof(double) * n, ctx->stream));
      c.dev.wdraw = c.dev.tot0 + kP0Vals;
    }
    c.dev.pstride0 = (int32_t)c.cap0;
    c.dev.pstride1 = (int32_t)c.cap1;
  }
  return BSG_OK;
}

// Block map of one colour for one chain: tiles of vpb voxels, at least one
// block per colour even when the colour has no voxels.  Colour 1's last
// arrival draws Omega; and the launch protocol relies on the colours
// alternating (a colour kernel's early phase reads its own colour's state,
// final once the other colour's kernel has passed its dependency point),
// so neither colour's launch may be left out.
void map_chain(std::vector<BlockMap> &m, int chain, int n, int vpb, int colour) {
  (void)colour;
  if (n == 0) m.push_back({(int32_t)chain, 0});
  for (int s = 0; s < n; s += vpb) m.push_back({(int32_t)chain, (int32_t)s});
}

// Rebuilds the device descriptor arrays and block maps.
bsg_status build_plan(bsg_ctx *ctx) {
  if (ctx->plan_valid) return BSG_OK;
  if (ctx->ch.empty()) return fail(ctx, BSG_ERR_STATE, "no chain");
  clear_graphs(ctx);
  cudaError_t e;
  if (ctx->d_ds_cap < ctx->ds.size()) {
    dfree(ctx, ctx->d_ds);
    ctx->d_ds_cap = ctx->ds.size() * 2;
    ctx->d_ds = (DatasetDev *)dalloc(ctx, sizeof(DatasetDev) * ctx->d_ds_cap, &e);
    CK(e);
  }
  if (ctx->d_ch_cap < ctx->ch.size()) {
    dfree(ctx, ctx->d_ch);
    ctx->d_ch_cap = ctx->ch.size() * 2;
    ctx->d_ch = (ChainDev *)dalloc(ctx, sizeof(ChainDev) * ctx->d_ch_cap, &e);
    CK(e);
  }
  const int vpb = ctx->threads / ctx->lpv;
  // partial rows for the smallest tile any kernel of this context uses
  bsg_status ps = ensure_partials(
      ctx, std::min({vpb, kParityThreads, ctx->threads / kMixLpv, kF64Threads}));
  if (ps) return ps;
  std::vector<DatasetDev> hds;
  for (auto &d : ctx->ds) hds.push_back(d.dev);
  std::vector<ChainDev> hch;
  for (auto &c : ctx->ch) hch.push_back(c.dev);
  CK(h2d(ctx, ctx->d_ds, hds.data(), sizeof(DatasetDev) * hds.size()));
  CK(h2d(ctx, ctx->d_ch, hch.data(), sizeof(ChainDev) * hch.size()));
  for (auto &g : ctx->groups) {
    for (int c = 0; c < 2; ++c) dfree(ctx, g.d_map[c]);
    for (auto &pr : g.pred) {
      dfree(ctx, pr.d_pmap);
      dfree(ctx, pr.d_fmap);
    }
  }
  ctx->groups.clear();
  for (size_t ci = 0; ci < ctx->ch.size(); ++ci) {
    const Dataset &d = ctx->ds[ctx->ch[ci].dataset];
    const bool mix = ctx->ch[ci].dev.model != 1;
    const bool wmu = ctx->ch[ci].dev.wm_update != 0;
    const bool f64 = ctx->ch[ci].dev.fp64 != 0;
    Group *g = nullptr;
    for (auto &gg : ctx->groups)
      if (gg.P == d.P && gg.mix == mix && gg.wm_any == wmu && gg.fp64 == f64) g = &gg;
    if (!g) {
      ctx->groups.push_back(Group());
      g = &ctx->groups.back();
      g->P = d.P;
      g->mix = mix;
      g->wm_any = wmu;
      g->fp64 = f64;
    }
    // the t/logit kernel runs kMixLpv lanes per voxel, the beta_WM one one,
    // the FP64 one one thread per voxel in blocks of kF64Threads
    const int gvpb = f64 ? kF64Threads
                         : (mix ? ctx->threads / kMixLpv : (wmu ? ctx->threads : vpb));
    for (int c = 0; c < 2; ++c) map_chain(g->map[c], (int)ci, (int)d.vox[c].size(), gvpb, c);
    g->vox += (double)d.V;
    g->subj_vox += (double)d.N * d.V;
    if (ctx->ch[ci].pred_on) {
      const ChainDev &cv = ctx->ch[ci].dev;
      Group::Pred *pr = nullptr;
      for (auto &q : g->pred)
        if (q.S == d.S) pr = &q;
      if (!pr) {
        g->pred.push_back(Group::Pred());
        pr = &g->pred.back();
        pr->S = d.S;
      }
      for (int t = 0; t < cv.pred_tiles; ++t) pr->pmap.push_back({(int32_t)ci, (int32_t)t});
      for (int b = 0; b * kPredWarps < d.N; ++b) pr->fmap.push_back({(int32_t)ci, (int32_t)b});
      pr->pchunks = std::max(pr->pchunks, (d.N + kPredThreads - 1) / kPredThreads);
    }
  }
  // The whole-word step of each probit / beta_WM group (one lane per
  // voxel): 16 subjects (four Philox calls at two resident blocks) where the
  // voxel's latent work dominates (P > 5, or N >= kWideMinN on average) or
  // the grid leaves SMs room (at most two blocks per SM), else 8 subjects
  // at three blocks; the results are the same either way.  Measured: the
  // 16-subject step is 6.5 % faster per sweep at N = 1000, P = 5 and 3.5 %
  // at N = 500, P = 6 (1.5M voxels); groups of 64 replicate studies with
  // N of 210-300 on average ran 2 % slower on it than on the 8-subject step.
  constexpr int kWideMinN = 384;
  int nsm = 0;
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
  for (auto &g : ctx->groups) {
    const bool eligible = !g.mix && !g.fp64 && (g.wm_any || (ctx->lpv == 1 && !ctx->tc));
    const bool fits = (int64_t)std::max(g.map[0].size(), g.map[1].size()) <= 2 * (int64_t)nsm;
    const bool auto_wide =
        g.P > 5 || g.subj_vox >= (double)kWideMinN * g.vox || fits;
    g.wide = eligible && (ctx->step == 16 || (ctx->step == 0 && auto_wide));
  }
  for (auto &g : ctx->groups) {
    for (int c = 0; c < 2; ++c) {
      g.d_map[c] = upload(ctx, g.map[c].data(), g.map[c].size(), &e);
      CK(e);
    }
    for (auto &pr : g.pred) {
      pr.d_pmap = upload(ctx, pr.pmap.data(), pr.pmap.size(), &e);
      CK(e);
      pr.d_fmap = upload(ctx, pr.fmap.data(), pr.fmap.size(), &e);
      CK(e);
    }
  }
  while (ctx->side.size() < ctx->groups.size()) {
    cudaStream_t s;
    cudaEvent_t ev;
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    ctx->side.push_back(s);
    ctx->join.push_back(ev);
  }
  ctx->plan_valid = true;
  return BSG_OK;
}

// Enqueues one sweep of every chain: per P group the two colour kernels
// (groups on parallel branches when there are several); the colour-1
// kernel also reduces the Omega pairs and draws Omega.
// One colour kernel of a group.
cudaError_t launch_colour(bsg_ctx *ctx, const Group &g, int c, cudaStream_t st, bool pdl) {
  if (g.fp64)
    return launch_fp64(g.P, ctx->d_ds, ctx->d_ch, g.d_map[c], (int)g.map[c].size(), c,
                       st);
  if (g.mix)
    return launch_fused_mix(g.P, ctx->threads, ctx->d_ds, ctx->d_ch, g.d_map[c],
                            (int)g.map[c].size(), c, st, pdl);
  if (g.wide)
    return launch_fused_wide(g.P, ctx->threads, g.wm_any, ctx->d_ds, ctx->d_ch, g.d_map[c],
                             (int)g.map[c].size(), c, st, pdl);
  if (g.wm_any)
    return launch_fused_wm(g.P, ctx->threads, ctx->d_ds, ctx->d_ch, g.d_map[c],
                           (int)g.map[c].size(), c, st, pdl);
  if (ctx->tc && ctx->lpv == 1)
    return launch_fused_tc(g.P, ctx->threads, ctx->d_ds, ctx->d_ch, g.d_map[c],
                           (int)g.map[c].size(), c, st, pdl);
  const Supplied sup{};
  return launch_fused(g.P, ctx->lpv, ctx->threads, false, ctx->d_ds, ctx->d_ch,
                      g.d_map[c], (int)g.map[c].size(), c, sup, st, pdl);
}

cudaError_t enqueue_group(bsg_ctx *ctx, const Group &g, cudaStream_t st) {
  cudaError_t e;
  for (int c = 0; c < 2; ++c) {
    // the colour-0 latent phase reads beta_WM, which the previous colour-1
    // kernel draws when the update is on: no early start then
    const bool pdl = ctx->pdl && !(c == 0 && g.wm_any) && !g.fp64;
    e = launch_colour(ctx, g, c, st, pdl);
    if (e != cudaSuccess) return e;
  }
  for (const auto &pr : g.pred) {
    // DIC / Qhat pass; its blocks return at once unless the sweep is kept
    e = launch_predict(g.P, pr.S, ctx->d_ds, ctx->d_ch, pr.d_pmap, (int)pr.pmap.size(),
                       pr.pchunks, 0, kPredKept, st, ctx->pdl);
    if (e != cudaSuccess) return e;
    e = launch_predict_finish(ctx->d_ds, ctx->d_ch, pr.d_fmap, (int)pr.fmap.size(), 0,
                              kPredKept, st, ctx->pdl);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t enqueue_sweep(bsg_ctx *ctx, cudaStream_t st) {
  cudaError_t e;
  if (ctx->groups.size() == 1) {
    if ((e = enqueue_group(ctx, ctx->groups[0], st)) != cudaSuccess) return e;
  } else {
    if ((e = cudaEventRecord(ctx->fork, st)) != cudaSuccess) return e;
    for (size_t gi = 0; gi < ctx->groups.size(); ++gi) {
      const Group &g = ctx->groups[gi];
      cudaStream_t s = ctx->side[gi];
      if ((e = cudaStreamWaitEvent(s, ctx->fork, 0)) != cudaSuccess) return e;
      if ((e = enqueue_group(ctx, g, s)) != cudaSuccess) return e;
      if ((e = cudaEventRecord(ctx->join[gi], s)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(st, ctx->join[gi], 0)) != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

bsg_status get_graph(bsg_ctx *ctx, int64_t nsw, cudaGraphExec_t *out) {
  auto it = ctx->graphs.find(nsw);
  if (it != ctx->graphs.end()) {
    *out = it->second;
    return BSG_OK;
  }
  cudaGraph_t graph = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int64_t s = 0; s < nsw && e == cudaSuccess; ++s) e = enqueue_sweep(ctx, ctx->stream);
  cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &graph);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return fail(ctx, BSG_ERR_CUDA,
                std::string("graph capture: ") +
                    cudaGetErrorString(e != cudaSuccess ? e : e2));
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  CK(e);
  ctx->graphs[nsw] = exec;
  *out = exec;
  return BSG_OK;
}

bool valid_chain(const bsg_ctx *ctx, int32_t c) {
  return ctx && c >= 0 && c < (int32_t)ctx->ch.size();
}


ChainCounters *counters_of(const Chain &c) {
  return reinterpret_cast<ChainCounters *>(c.dev.sweep);  // first member
}

PredCounters *pred_counters_of(const Chain &c) {
  return reinterpret_cast<PredCounters *>(c.dev.npred);  // first member
}

// Buffers of the predictive pass, allocated on first use (zeroed).
bsg_status ensure_pred(bsg_ctx *ctx, Chain &c) {
  if (c.dev.pred_part) return BSG_OK;
  const Dataset &d = ctx->ds[c.dataset];
  // Tiles sized so that one chain's grid (tiles x subject chunks) is about
  // one wave of resident blocks.
  const int ntot = (int)(d.vox[0].size() + d.vox[1].size());
  const int chunks = (d.N + kPredThreads - 1) / kPredThreads;
  int sms = 1;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const int cap = sms * predict_blocks_per_sm(d.P, std::max(d.S, 1));
  const int want = std::max(1, cap / std::max(chunks, 1));
  int tile = (ntot + want - 1) / want;
  tile = std::max(kPredThreads, (tile + kPredThreads - 1) / kPredThreads * kPredThreads);
  const int T = std::max(1, (ntot + tile - 1) / tile);
  const size_t N = (size_t)d.N, G = (size_t)std::max(d.S, 1);
  cudaError_t e;
  ChainDev &cv = c.dev;
  double *part = (double *)dalloc(ctx, sizeof(double) * T * N * G, &e);
  CK(e);
  cv.pred_subj = (double *)dalloc(ctx, sizeof(double) * N, &e);
  CK(e);
  cv.mpred = (double *)dalloc(ctx, sizeof(double) * N * G, &e);
  CK(e);
  cv.qhat = (double *)dalloc(ctx, sizeof(double) * N * G, &e);
  CK(e);
  cv.pred_sums = (double *)dalloc(ctx, sizeof(double) * 2, &e);
  CK(e);
  PredCounters *pc = (PredCounters *)dalloc(ctx, sizeof(PredCounters), &e);
  CK(e);
  CK(cudaMemsetAsync(cv.mpred, 0, sizeof(double) * N * G, ctx->stream));
  CK(cudaMemsetAsync(cv.qhat, 0, sizeof(double) * N * G, ctx->stream));
  CK(cudaMemsetAsync(cv.pred_sums, 0, sizeof(double) * 2, ctx->stream));
  CK(cudaMemsetAsync(pc, 0, sizeof(PredCounters), ctx->stream));
  cv.npred = &pc->npred;
  cv.pred_done = &pc->done;
  cv.pred_tiles = T;
  cv.pred_tile = tile;
  cv.pred_part = part;
  ctx->plan_valid = false;  // the device copy of the chain changed
  return BSG_OK;
}

// Link of a chain (the reference's MODEL and its t_df / logit_factor,
// main.cu:42,168-175).  The t/logit links start from weights phi = 1.
bsg_status set_model(bsg_ctx *ctx, Chain &c, int model) {
  const Dataset &d = ctx->ds[c.dataset];
  ChainDev &cv = c.dev;
  cudaError_t e;
  if (model != 1) {
    for (int k = 0; k < 2; ++k) {
      const size_t n = (size_t)d.N * d.vox[k].size();
      if (!cv.phi[k]) {
        cv.phi[k] = (float *)dalloc(ctx, sizeof(float) * (n ? n : 1), &e);
        CK(e);
      }
      CK(launch_fill(cv.phi[k], n, 1.0f, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
  }
  cv.model = model;
  cv.t_df = model == 0 ? 8.f : (model == 2 ? 3.f : 1000.f);
  cv.inv_lf = model == 0 ? (float)(1.0 / 0.634) : 1.f;
  const double alpha = 0.5 * ((double)cv.t_df + 1.0), dd = alpha - 1.0 / 3.0;
  cv.mix_d = (float)dd;
  cv.mix_c = (float)(1.0 / std::sqrt(9.0 * dd));
  ctx->plan_valid = false;
  return BSG_OK;
}

// Turns a chain's FP64 mode on or off.  On: the FP64 coefficients start
// from the current float ones.  Off: the float copy (kept in step by the
// FP64 kernel) simply carries on.
bsg_status set_precision(bsg_ctx *ctx, Chain &c, int bits) {
  const Dataset &d = ctx->ds[c.dataset];
  const size_t n = (size_t)d.P * d.Vp;
  cudaError_t e;
  if (bits == 64) {
    if (!c.dev.beta64) {
      c.dev.beta64 = (double *)dalloc(ctx, sizeof(double) * n, &e);
      CK(e);
    }
    std::vector<float> bf(n);
    CK(d2h(ctx, bf.data(), c.dev.beta, sizeof(float) * n));
    std::vector<double> bd(bf.begin(), bf.end());
    CK(h2d(ctx, c.dev.beta64, bd.data(), sizeof(double) * n));
  }
  const int32_t on = bits == 64 ? 1 : 0;
  if (c.dev.fp64 != on) ctx->plan_valid = false;
  c.dev.fp64 = on;
  return BSG_OK;
}
}  // namespace

// ========================================================================
extern "C" {

const char *bsg_status_string(bsg_status s) {
  switch (s) {
    case BSG_OK: return "ok";
    case BSG_ERR_INVALID: return "invalid argument";
    case BSG_ERR_CUDA: return "CUDA error";
    case BSG_ERR_NOT_SPD: return "matrix not positive definite";
    case BSG_ERR_SAMPLER_CAP: return "sampler iteration cap reached";
    case BSG_ERR_NAN: return "non-finite sampler state";
    case BSG_ERR_STATE: return "call out of order";
    case BSG_ERR_NO_DEVICE: return "no CUDA device";
    case BSG_ERR_UNSUPPORTED: return "unsupported size";
    default: return "unknown status";
  }
}

const char *bsg_last_error(const bsg_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }

bsg_status bsg_create(int32_t device, bsg_ctx **out) {
  if (!out) return BSG_ERR_INVALID;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return BSG_ERR_NO_DEVICE;
  if (device < 0 || device >= n) return BSG_ERR_INVALID;
  std::unique_ptr<bsg_ctx> c(new bsg_ctx());
  bsg_ctx *ctx = c.get();
  ctx->device = device;
  CK(cudaSetDevice(device));
  CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming));
  *out = c.release();
  return BSG_OK;
}

bsg_status bsg_destroy(bsg_ctx *ctx) {
  if (!ctx) return BSG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  clear_graphs(ctx);
  for (auto &b : ctx->owned) cudaFree(b.p);
  for (auto s : ctx->side) cudaStreamDestroy(s);
  for (auto e : ctx->join) cudaEventDestroy(e);
  if (ctx->fork) cudaEventDestroy(ctx->fork);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->pin) cudaFreeHost(ctx->pin);
  delete ctx;
  return BSG_OK;
}

bsg_status bsg_add_dataset(bsg_ctx *ctx, const bsg_dataset_desc *desc,
                           int32_t *dataset_id) {
  if (!ctx || !desc || !dataset_id) return BSG_ERR_INVALID;
  const bsg_dataset_desc &q = *desc;
  if (q.nrow < 1 || q.ncol < 1 || q.ndepth < 1 || !q.mask || !q.covar || !q.data)
    return fail(ctx, BSG_ERR_INVALID, "dataset: empty grid or null input");
  const double padded = (double)(q.nrow + 2) * (q.ncol + 2) * (q.ndepth + 2);
  if (padded > 2.0e9) return fail(ctx, BSG_ERR_UNSUPPORTED, "grid too large");
  if (q.ncovar < 1 || q.ncovar > BSG_MAX_COVAR)
    return fail(ctx, BSG_ERR_UNSUPPORTED, "ncovar must be in 1..8");
  if (q.nsubtypes < 0 || q.nsubtypes > q.ncovar)
    return fail(ctx, BSG_ERR_INVALID, "nsubtypes must be in 0..ncovar");
  if (q.nsubs < 1 || q.nsubs > (1 << 26))
    return fail(ctx, BSG_ERR_INVALID, "nsubs out of range");
  CK(cudaSetDevice(ctx->device));
  Dataset d;
  d.X = q.nrow;
  d.Y = q.ncol;
  d.Z = q.ndepth;
  d.N = q.nsubs;
  d.P = q.ncovar;
  d.S = q.nsubtypes;
  build_lattice(d, q.mask);
  if (d.V == 0) return fail(ctx, BSG_ERR_INVALID, "mask is empty");
  if ((double)d.N * d.V > 4.0e12)
    return fail(ctx, BSG_ERR_UNSUPPORTED, "N*V too large");
  // X'X in float, subject order (read_data.cpp:321-327).
  std::vector<float> xtx((size_t)d.P * d.P, 0.f);
  for (int i = 0; i < d.N; ++i)
    for (int a = 0; a < d.P; ++a)
      for (int b = 0; b < d.P; ++b)
        xtx[b + a * d.P] += q.covar[(size_t)a * d.N + i] * q.covar[(size_t)b * d.N + i];
  cudaError_t e;
  DatasetDev &dv = d.dev;
  dv.N = d.N;
  dv.P = d.P;
  dv.S = d.S;
  dv.V = d.V;
  dv.Vp = d.Vp;
  dv.W = (d.N + 31) / 32;
  dv.covar = upload(ctx, q.covar, (size_t)d.P * d.N, &e);
  CK(e);
  dv.xtx = upload(ctx, xtx.data(), xtx.size(), &e);
  CK(e);
  dv.wm = nullptr;
  if (q.wm) {
    dv.wm = upload(ctx, q.wm, (size_t)d.V, &e);
    CK(e);
  }
  // For the beta_WM update: column sums of X, c with X c = 1 (least
  // squares, kept if the fit is exact to 1e-4: an intercept or group
  // indicators that cover every subject), and sum_v WM_v^2.
  {
    const int P = d.P, N = d.N;
    std::vector<double> A((size_t)P * P, 0.0), rhs(P, 0.0);
    for (int i = 0; i < N; ++i)
      for (int a = 0; a < P; ++a) {
        const double xa = q.covar[(size_t)a * N + i];
        rhs[a] += xa;
        for (int b2 = 0; b2 < P; ++b2) A[a * P + b2] += xa * q.covar[(size_t)b2 * N + i];
      }
    std::vector<float> xsum(P), cvec(P, 0.f);
    for (int a = 0; a < P; ++a) xsum[a] = (float)rhs[a];
    std::vector<double> c = rhs;
    bool ok = true;  // Gaussian elimination with partial pivoting
    std::vector<double> M = A;
    for (int k = 0; k < P && ok; ++k) {
      int piv = k;
      for (int r = k + 1; r < P; ++r)
        if (std::fabs(M[r * P + k]) > std::fabs(M[piv * P + k])) piv = r;
      if (!(std::fabs(M[piv * P + k]) > 1e-12 * (1.0 + std::fabs(A[k * P + k])))) {
        ok = false;
        break;
      }
      if (piv != k) {
        for (int t = 0; t < P; ++t) std::swap(M[k * P + t], M[piv * P + t]);
        std::swap(c[k], c[piv]);
      }
      for (int r = k + 1; r < P; ++r) {
        const double f = M[r * P + k] / M[k * P + k];
        for (int t = k; t < P; ++t) M[r * P + t] -= f * M[k * P + t];
        c[r] -= f * c[k];
      }
    }
    if (ok) {
      for (int k = P - 1; k >= 0; --k) {
        double t = c[k];
        for (int u = k + 1; u < P; ++u) t -= M[k * P + u] * c[u];
        c[k] = t / M[k * P + k];
      }
      for (int i = 0; i < N && ok; ++i) {
        double f = 0.0;
        for (int a = 0; a < P; ++a) f += c[a] * q.covar[(size_t)a * N + i];
        ok = std::fabs(f - 1.0) < 1e-4;
      }
    }
    dv.has_c = ok ? 1 : 0;
    if (ok)
      for (int a = 0; a < P; ++a) cvec[a] = (float)c[a];
    dv.xsum = upload(ctx, xsum.data(), xsum.size(), &e);
    CK(e);
    dv.cvec = upload(ctx, cvec.data(), cvec.size(), &e);
    CK(e);
    double w2 = 0.0;
    for (int v = 0; v < d.V; ++v) {
      const double w = q.wm ? (double)q.wm[v] : 1.0;
      w2 += w * w;
    }
    dv.wm2 = w2;
  }
  uint8_t *bytes = upload(ctx, q.data, (size_t)d.N * d.V, &e);
  CK(e);
  int *status = (int *)dalloc(ctx, sizeof(int), &e);
  CK(e);
  CK(cudaMemsetAsync(status, 0, sizeof(int), ctx->stream));
  const int sy = d.PX, sz = d.PX * d.PY;
  const int off[6] = {-1, 1, -sy, sy, -sz, sz};
  for (int c = 0; c < 2; ++c) {
    const int nc = (int)d.vox[c].size();
    dv.n[c] = nc;
    std::vector<int32_t> nb((size_t)7 * nc), vi(nc);
    for (int j = 0; j < nc; ++j) {
      const int p = d.vox[c][j];
      nb[j] = d.idxsc[p];
      for (int t = 0; t < 6; ++t) nb[(size_t)(t + 1) * nc + j] = d.idxsc[p + off[t]];
      vi[j] = d.idx[p];
    }
    dv.nb[c] = upload(ctx, nb.data(), nb.size(), &e);
    CK(e);
    std::vector<uint8_t> nbm(nc);
    for (int j = 0; j < nc; ++j) {
      const int p = d.vox[c][j];
      unsigned m = 0;
      for (int t = 0; t < 6; ++t) m |= (d.idx[p + off[t]] >= 0 ? 1u : 0u) << t;
      nbm[j] = (uint8_t)m;
    }
    dv.nbm[c] = upload(ctx, nbm.data(), nbm.size(), &e);
    CK(e);
    dv.vidx[c] = upload(ctx, vi.data(), vi.size(), &e);
    CK(e);
    uint32_t *yb = (uint32_t *)dalloc(ctx, sizeof(uint32_t) * (size_t)dv.W * nc, &e);
    CK(e);
    dv.ybits[c] = yb;
    CK(launch_pack(bytes, d.N, d.V, nc, dv.vidx[c], yb, status, ctx->stream));
  }
  int bad = 0;
  CK(d2h(ctx, &bad, status, sizeof(int)));
  CK(cudaStreamSynchronize(ctx->stream));
  dfree(ctx, bytes);
  dfree(ctx, status);
  if (bad) return fail(ctx, BSG_ERR_INVALID, "outcome values must be 0 or 1");
  ctx->ds.push_back(std::move(d));
  *dataset_id = (int32_t)ctx->ds.size() - 1;
  ctx->plan_valid = false;
  return BSG_OK;
}

bsg_status bsg_add_chain(bsg_ctx *ctx, int32_t dataset_id,
                         const bsg_chain_desc *desc, int32_t *chain_id) {
  if (!ctx || !desc || !chain_id) return BSG_ERR_INVALID;
  if (dataset_id < 0 || dataset_id >= (int32_t)ctx->ds.size())
    return fail(ctx, BSG_ERR_INVALID, "no such dataset");
  if (desc->thin < 1) return fail(ctx, BSG_ERR_INVALID, "thin must be >= 1");
  if (ctx->ch.size() >= (1u << 23))
    return fail(ctx, BSG_ERR_UNSUPPORTED, "too many chains");
  const Dataset &d = ctx->ds[dataset_id];
  if ((double)d.V + desc->df_offset < d.P)
    return fail(ctx, BSG_ERR_INVALID, "Wishart df = V + df_offset must be >= P");
  CK(cudaSetDevice(ctx->device));
  Chain c;
  c.dataset = dataset_id;
  c.desc = *desc;
  ChainDev &cv = c.dev;
  cudaError_t e;
  cv.dataset = dataset_id;
  cv.key0 = (uint32_t)(desc->seed & 0xFFFFFFFFu);
  cv.key1 = (uint32_t)(desc->seed >> 32);
  cv.chain_id = (uint32_t)ctx->ch.size();
  cv.wm_update = 0;
  cv.model = 1;  // probit (main.cu:42)
  cv.t_df = 1000.f;
  cv.inv_lf = 1.f;
  cv.df_offset = desc->df_offset;
  cv.burnin = desc->burnin;
  cv.thin = desc->thin;
  const int P = d.P;
  cv.beta = (float *)dalloc(ctx, sizeof(float) * (size_t)P * d.Vp, &e);
  CK(e);
  CK(cudaMemsetAsync(cv.beta, 0, sizeof(float) * (size_t)P * d.Vp, ctx->stream));
  std::vector<double> eye((size_t)P * P, 0.0);
  std::vector<float> eyef((size_t)P * P, 0.f);
  for (int i = 0; i < P; ++i) eye[i + i * P] = 1.0, eyef[i + i * P] = 1.f;
  cv.omega_d = upload(ctx, eye.data(), eye.size(), &e);
  CK(e);
  cv.omega_f = upload(ctx, eyef.data(), eyef.size(), &e);
  CK(e);
  cv.colmean = (float *)dalloc(ctx, sizeof(float) * P, &e);
  CK(e);
  WmState *wst = (WmState *)dalloc(ctx, sizeof(WmState), &e);
  CK(e);
  const WmState w0{0.0, desc->beta_wm, 0};
  CK(h2d(ctx, wst, &w0, sizeof(w0)));
  cv.wm_sum = &wst->sum;
  cv.wm_beta = &wst->beta;
  CK(cudaMemsetAsync(cv.colmean, 0, sizeof(float) * P, ctx->stream));
  const size_t nacc = (size_t)P * d.V, nprb = (size_t)d.S * d.V;
  cv.acc_sum = (double *)dalloc(ctx, sizeof(double) * nacc, &e);
  CK(e);
  cv.acc_sq = (double *)dalloc(ctx, sizeof(double) * nacc, &e);
  CK(e);
  cv.prb_sum = (double *)dalloc(ctx, sizeof(double) * (nprb ? nprb : 1), &e);
  CK(e);
  CK(cudaMemsetAsync(cv.acc_sum, 0, sizeof(double) * nacc, ctx->stream));
  CK(cudaMemsetAsync(cv.acc_sq, 0, sizeof(double) * nacc, ctx->stream));
  if (nprb) CK(cudaMemsetAsync(cv.prb_sum, 0, sizeof(double) * nprb, ctx->stream));
  ChainCounters *cnt = (ChainCounters *)dalloc(ctx, sizeof(ChainCounters), &e);
  CK(e);
  CK(cudaMemsetAsync(cnt, 0, sizeof(ChainCounters), ctx->stream));
  cv.sweep = cnt->sweep;
  cv.nkept = &cnt->nkept;
  cv.done = cnt->done;
  cv.status = &cnt->status;
  if (!ctx->any_status) {
    ctx->any_status = (int *)dalloc(ctx, sizeof(int), &e);
    CK(e);
    CK(cudaMemsetAsync(ctx->any_status, 0, sizeof(int), ctx->stream));
  }
  cv.any_status = ctx->any_status;
  ctx->ch.push_back(c);
  *chain_id = (int32_t)ctx->ch.size() - 1;
  ctx->plan_valid = false;
  return BSG_OK;
}

bsg_status bsg_set_tuning(bsg_ctx *ctx, int32_t lanes_per_voxel,
                          int32_t block_threads) {
  if (!ctx) return BSG_ERR_INVALID;
  const int lpv = lanes_per_voxel ? lanes_per_voxel : ctx->lpv;
  const int thr = block_threads ? block_threads : ctx->threads;
  if (!fused_supported(1, lpv, thr))
    return fail(ctx, BSG_ERR_UNSUPPORTED,
                "lanes_per_voxel in {1,2,4,8}, block_threads in {64,128,256}");
  if (lpv != ctx->lpv || thr != ctx->threads) {
    ctx->lpv = lpv;
    ctx->threads = thr;
    ctx->plan_valid = false;
  }
  return BSG_OK;
}

bsg_status bsg_set_tensor_xz(bsg_ctx *ctx, int32_t enable) {
  if (!ctx) return BSG_ERR_INVALID;
  const bool on = enable != 0;
  if (on != ctx->tc) {
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    if (on) CK(prepare_fused_tc());
    clear_graphs(ctx);  // the segments hold the other kernel
    ctx->tc = on;
  }
  return BSG_OK;
}

bsg_status bsg_set_step_subjects(bsg_ctx *ctx, int32_t subjects) {
  if (!ctx) return BSG_ERR_INVALID;
  if (subjects != 0 && subjects != 8 && subjects != 16)
    return fail(ctx, BSG_ERR_UNSUPPORTED, "subjects per step in {0 (per group), 8, 16}");
  if (subjects != ctx->step) {
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    clear_graphs(ctx);  // the segments hold the other kernels
    ctx->step = subjects;
    ctx->plan_valid = false;
  }
  return BSG_OK;
}

bsg_status bsg_get_step_subjects(bsg_ctx *ctx, int32_t *subjects) {
  if (!ctx || !subjects) return BSG_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  bsg_status s = build_plan(ctx);
  if (s) return s;
  int n = 0;
  for (const auto &g : ctx->groups)
    if (!g.mix && !g.fp64) n = std::max(n, g.wide ? 16 : 8);
  *subjects = n;
  return BSG_OK;
}

bsg_status bsg_get_tuning(const bsg_ctx *ctx, int32_t *lpv, int32_t *thr) {
  if (!ctx) return BSG_ERR_INVALID;
  if (lpv) *lpv = ctx->lpv;
  if (thr) *thr = ctx->threads;
  return BSG_OK;
}

bsg_status bsg_run(bsg_ctx *ctx, int64_t nsweeps) {
  if (!ctx || nsweeps < 0) return BSG_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  bsg_status s = build_plan(ctx);
  if (s) return s;
  int64_t left = nsweeps;
  while (left > 0) {
    int64_t seg = 64;
    while (seg > left) seg >>= 1;
    cudaGraphExec_t g;
    if ((s = get_graph(ctx, seg, &g))) return s;
    CK(cudaGraphLaunch(g, ctx->stream));
    left -= seg;
  }
  return BSG_OK;
}

bsg_status bsg_sync(bsg_ctx *ctx) {
  if (!ctx) return BSG_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  int bits = 0;
  if (ctx->any_status)
    CK(d2h(ctx, &bits, ctx->any_status, sizeof(int)));
  if (bits) {
    ctx->err = "sampler:" + status_text(bits);
    for (size_t i = 0; i < ctx->ch.size(); ++i) {
      int b = 0;
      CK(d2h(ctx, &b, ctx->ch[i].dev.status, sizeof(int)));
      if (b) ctx->err += " (chain " + std::to_string(i) + ")";
    }
    return status_from_bits(bits);
  }
  return BSG_OK;
}

bsg_status bsg_step_host(bsg_ctx *ctx, int32_t chain, const double *omega_in,
                         int64_t nsweeps, double *omega_out, float *colmeans_out) {
  if (!valid_chain(ctx, chain) || nsweeps < 0) return BSG_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  bsg_status s = build_plan(ctx);
  if (s) return s;
  const Chain &c = ctx->ch[chain];
  const int P = ctx->ds[c.dataset].P;
  // staging: Omega in (FP64, FP32), Omega out, column means, status word
  const size_t nd = sizeof(double) * P * P, nf = sizeof(float) * P * P;
  const size_t need = 2 * nd + nf + sizeof(float) * P + sizeof(int);
  if (ctx->pin_busy) {  // a previous call returned before its copies finished
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->pin_busy = false;
  }
  if (ctx->pin_bytes < need) {
    if (ctx->pin) CK(cudaFreeHost(ctx->pin));
    ctx->pin = nullptr;
    ctx->pin_bytes = 0;
    CK(cudaHostAlloc(&ctx->pin, need, cudaHostAllocDefault));
    ctx->pin_bytes = need;
  }
  char *base = (char *)ctx->pin;
  double *in_d = (double *)base, *out_d = (double *)(base + nd);
  float *in_f = (float *)(base + 2 * nd), *cm = (float *)(base + 2 * nd + nf);
  int *bits = (int *)(base + 2 * nd + nf + sizeof(float) * P);
  ctx->pin_busy = true;
  if (omega_in) {
    for (int i = 0; i < P * P; ++i) {
      in_d[i] = omega_in[i];
      in_f[i] = (float)omega_in[i];
    }
    CK(cudaMemcpyAsync(c.dev.omega_d, in_d, nd, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(c.dev.omega_f, in_f, nf, cudaMemcpyHostToDevice, ctx->stream));
  }
  if (nsweeps > 0 && (s = bsg_run(ctx, nsweeps))) return s;
  if (omega_out)
    CK(cudaMemcpyAsync(out_d, c.dev.omega_d, nd, cudaMemcpyDeviceToHost, ctx->stream));
  if (colmeans_out)
    CK(cudaMemcpyAsync(cm, c.dev.colmean, sizeof(float) * P, cudaMemcpyDeviceToHost,
                       ctx->stream));
  *bits = 0;
  if (ctx->any_status)
    CK(cudaMemcpyAsync(bits, ctx->any_status, sizeof(int), cudaMemcpyDeviceToHost,
                       ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->pin_busy = false;
  if (*bits) return bsg_sync(ctx);  // names the failing chains
  if (omega_out) std::memcpy(omega_out, out_d, nd);
  if (colmeans_out) std::memcpy(colmeans_out, cm, sizeof(float) * P);
  return BSG_OK;
}

bsg_status bsg_run_timed(bsg_ctx *ctx, int64_t nsweeps, double *ms) {
  if (!ctx || !ms) return BSG_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  bsg_status s = build_plan(ctx);
  if (s) return s;
  // Warm the graph cache outside the timed region.
  int64_t left = nsweeps;
  while (left > 0) {
    int64_t seg = 64;
    while (seg > left) seg >>= 1;
    cudaGraphExec_t g;
    if ((s = get_graph(ctx, seg, &g))) return s;
    left -= seg;
  }
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(cudaEventRecord(a, ctx->stream));
  s = bsg_run(ctx, nsweeps);
  CK(cudaEventRecord(b, ctx->stream));
  CK(cudaEventSynchronize(b));
  float f = 0.f;
  CK(cudaEventElapsedTime(&f, a, b));
  *ms = f;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return s;
}

bsg_status bsg_profile(bsg_ctx *ctx, int64_t nsweeps, double *ms,
                       int64_t *launches) {
  if (!ctx || !ms || nsweeps < 0) return BSG_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  bsg_status s = build_plan(ctx);
  if (s) return s;
  std::vector<cudaEvent_t> ev((size_t)3 * nsweeps);
  for (auto &e : ev) CK(cudaEventCreate(&e));
  int64_t nl[3] = {0, 0, 0};
  for (int64_t i = 0; i < nsweeps; ++i) {
    for (int c = 0; c < 2; ++c) {
      CK(cudaEventRecord(ev[3 * i + c], ctx->stream));
      for (const Group &g : ctx->groups) {
        CK(launch_colour(ctx, g, c, ctx->stream, false));
        nl[c]++;
      }
    }
    nl[2]++;
    CK(cudaEventRecord(ev[3 * i + 2], ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  double t[3] = {0, 0, 0};
  for (int64_t i = 0; i < nsweeps; ++i) {
    float a = 0, b = 0, c = 0;
    CK(cudaEventElapsedTime(&a, ev[3 * i], ev[3 * i + 1]));
    CK(cudaEventElapsedTime(&b, ev[3 * i + 1], ev[3 * i + 2]));
    CK(cudaEventElapsedTime(&c, ev[3 * i], ev[3 * i + 2]));
    t[0] += a;
    t[1] += b;
    t[2] += c;
  }
  for (auto &e : ev) cudaEventDestroy(e);
  for (int i = 0; i < 3; ++i) {
    ms[i] = t[i];
    if (launches) launches[i] = nl[i];
  }
  return BSG_OK;
}

int64_t bsg_launches_per_sweep(const bsg_ctx *ctx) {
  if (!ctx) return 0;
  std::vector<int> ps, pp;
  for (auto &c : ctx->ch) {
    const Dataset &d = ctx->ds[c.dataset];
    const int P = d.P * 8 + (c.dev.model != 1) * 2 + (c.dev.wm_update != 0) +
                  (c.dev.fp64 != 0) * 4;
    const int PS = d.P * 16 + d.S;
    if (std::find(ps.begin(), ps.end(), P) == ps.end()) ps.push_back(P);
    if (c.pred_on && std::find(pp.begin(), pp.end(), PS) == pp.end()) pp.push_back(PS);
  }
  return (int64_t)(2 * ps.size() + 2 * pp.size());
}

void *bsg_stream(bsg_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

bsg_status bsg_dataset_info(const bsg_ctx *ctx, int32_t id, int64_t *info) {
  if (!ctx || !info || id < 0 || id >= (int32_t)ctx->ds.size()) return BSG_ERR_INVALID;
  const Dataset &d = ctx->ds[id];
  const int64_t v[11] = {d.X, d.Y, d.Z, d.nsize, d.V, d.Vp,
                         (int64_t)d.vox[0].size(), (int64_t)d.vox[1].size(),
                         d.N, d.P, d.S};
  std::memcpy(info, v, sizeof(v));
  return BSG_OK;
}

bsg_status bsg_get_lattice(const bsg_ctx *ctx, int32_t id, int32_t *idx,
                           int32_t *idxsc, int32_t *vox0, int32_t *vox1,
                           uint8_t *nbrs0, uint8_t *nbrs1) {
  if (!ctx || id < 0 || id >= (int32_t)ctx->ds.size()) return BSG_ERR_INVALID;
  const Dataset &d = ctx->ds[id];
  if (idx) std::memcpy(idx, d.idx.data(), sizeof(int32_t) * d.nsize);
  if (idxsc) std::memcpy(idxsc, d.idxsc.data(), sizeof(int32_t) * d.nsize);
  if (vox0) std::memcpy(vox0, d.vox[0].data(), sizeof(int32_t) * d.vox[0].size());
  if (vox1) std::memcpy(vox1, d.vox[1].data(), sizeof(int32_t) * d.vox[1].size());
  if (nbrs0) std::memcpy(nbrs0, d.nbrs[0].data(), d.nbrs[0].size());
  if (nbrs1) std::memcpy(nbrs1, d.nbrs[1].data(), d.nbrs[1].size());
  return BSG_OK;
}

bsg_status bsg_get_beta(bsg_ctx *ctx, int32_t chain, float *out) {
  if (!valid_chain(ctx, chain) || !out) return BSG_ERR_INVALID;
  const Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  CK(cudaSetDevice(ctx->device));
  CK(d2h(ctx, out, c.dev.beta, sizeof(float) * (size_t)d.P * d.Vp));
  return BSG_OK;
}

bsg_status bsg_set_beta(bsg_ctx *ctx, int32_t chain, const float *in) {
  if (!valid_chain(ctx, chain) || !in) return BSG_ERR_INVALID;
  const Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  // Entries outside the mask (the dilated border) must stay zero: they are
  // the out-of-mask neighbours (covarGPU.cu:357-362).
  std::vector<float> b(in, in + (size_t)d.P * d.Vp);
  std::vector<char> inmask(d.Vp, 0);
  for (int p = 0; p < d.nsize; ++p)
    if (d.idx[p] >= 0) inmask[d.idxsc[p]] = 1;
  for (int p = 0; p < d.P; ++p)
    for (int s = 0; s < d.Vp; ++s)
      if (!inmask[s]) b[(size_t)p * d.Vp + s] = 0.f;
  CK(cudaSetDevice(ctx->device));
  CK(h2d(ctx, c.dev.beta, b.data(), sizeof(float) * b.size()));
  if (c.dev.fp64) {  // the FP64 chain's own coefficients follow
    std::vector<double> bd(b.begin(), b.end());
    CK(h2d(ctx, c.dev.beta64, bd.data(), sizeof(double) * bd.size()));
  }
  return BSG_OK;
}

bsg_status bsg_get_omega(bsg_ctx *ctx, int32_t chain, double *out) {
  if (!valid_chain(ctx, chain) || !out) return BSG_ERR_INVALID;
  const Chain &c = ctx->ch[chain];
  const int P = ctx->ds[c.dataset].P;
  CK(cudaSetDevice(ctx->device));
  CK(d2h(ctx, out, c.dev.omega_d, sizeof(double) * P * P));
  return BSG_OK;
}

bsg_status bsg_set_omega(bsg_ctx *ctx, int32_t chain, const double *in) {
  if (!valid_chain(ctx, chain) || !in) return BSG_ERR_INVALID;
  const Chain &c = ctx->ch[chain];
  const int P = ctx->ds[c.dataset].P;
  std::vector<float> f(in, in + P * P);
  CK(cudaSetDevice(ctx->device));
  CK(h2d(ctx, c.dev.omega_d, in, sizeof(double) * P * P));
  CK(h2d(ctx, c.dev.omega_f, f.data(), sizeof(float) * P * P));
  return BSG_OK;
}

bsg_status bsg_set_beta_wm(bsg_ctx *ctx, int32_t chain, float beta_wm) {
  if (!valid_chain(ctx, chain) || !std::isfinite(beta_wm)) return BSG_ERR_INVALID;
  Chain &c = ctx->ch[chain];
  c.desc.beta_wm = beta_wm;
  CK(cudaSetDevice(ctx->device));
  CK(h2d(ctx, c.dev.wm_beta, &beta_wm, sizeof(float)));
  CK(cudaStreamSynchronize(ctx->stream));
  return BSG_OK;
}

bsg_status bsg_set_wm_update(bsg_ctx *ctx, int32_t chain, int32_t enable) {
  if (!valid_chain(ctx, chain)) return BSG_ERR_INVALID;
  Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  if (enable && !d.dev.has_c)
    return fail(ctx, BSG_ERR_UNSUPPORTED,
                "the beta_WM update needs design columns that sum to 1 for every "
                "subject (an intercept or a full set of group indicators)");
  if (enable && !(d.dev.wm2 > 0.0))
    return fail(ctx, BSG_ERR_INVALID, "the beta_WM update needs a nonzero WM map");
  if (enable && c.dev.model != 1)
    return fail(ctx, BSG_ERR_UNSUPPORTED, "the beta_WM update is probit only");
  if (enable && c.dev.fp64)
    return fail(ctx, BSG_ERR_UNSUPPORTED, "FP64 chains keep beta_WM fixed");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  const int32_t on = enable ? 1 : 0;
  if (c.dev.wm_update != on) ctx->plan_valid = false;
  c.dev.wm_update = on;
  return BSG_OK;
}

bsg_status bsg_get_beta_wm(bsg_ctx *ctx, int32_t chain, float *beta_wm,
                           double *mean_kept) {
  if (!valid_chain(ctx, chain)) return BSG_ERR_INVALID;
  const Chain &c = ctx->ch[chain];
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  WmState w{};
  CK(d2h(ctx, &w, c.dev.wm_sum, sizeof(w)));
  long long nk = 0;
  CK(d2h(ctx, &nk, c.dev.nkept, sizeof(nk)));
  if (beta_wm) *beta_wm = w.beta;
  if (mean_kept) *mean_kept = nk > 0 ? w.sum / (double)nk : 0.0;
  return BSG_OK;
}

bsg_status bsg_get_colmeans(bsg_ctx *ctx, int32_t chain, float *out) {
  if (!valid_chain(ctx, chain) || !out) return BSG_ERR_INVALID;
  const Chain &c = ctx->ch[chain];
  CK(cudaSetDevice(ctx->device));
  CK(d2h(ctx, out, c.dev.colmean, sizeof(float) * ctx->ds[c.dataset].P));
  return BSG_OK;
}

bsg_status bsg_get_sweep(bsg_ctx *ctx, int32_t chain, int64_t *sweep, int64_t *nkept) {
  if (!valid_chain(ctx, chain)) return BSG_ERR_INVALID;
  ChainCounters h{};
  CK(cudaSetDevice(ctx->device));
  CK(d2h(ctx, &h, counters_of(ctx->ch[chain]), sizeof(h)));
  if (sweep) *sweep = h.sweep[1];
  if (nkept) *nkept = h.nkept;
  return BSG_OK;
}

bsg_status bsg_compute_prb(bsg_ctx *ctx, int32_t chain, float *prb) {
  if (!valid_chain(ctx, chain) || !prb) return BSG_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  bsg_status s = build_plan(ctx);
  if (s) return s;
  const Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  const size_t n = (size_t)d.S * d.V;
  if (!n) return BSG_OK;
  cudaError_t e;
  float *dp = (float *)dalloc(ctx, sizeof(float) * n, &e);
  CK(e);
  CK(launch_prb(ctx->d_ds, ctx->d_ch, chain, d.dev, dp, ctx->stream));
  CK(d2h(ctx, prb, dp, sizeof(float) * n));
  CK(cudaStreamSynchronize(ctx->stream));
  dfree(ctx, dp);
  return BSG_OK;
}

bsg_status bsg_get_posterior(bsg_ctx *ctx, int32_t chain, double *mean,
                             double *var, double *prb, int64_t *nkept) {
  if (!valid_chain(ctx, chain)) return BSG_ERR_INVALID;
  const Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  int64_t nk = 0;
  bsg_status s = bsg_get_sweep(ctx, chain, nullptr, &nk);
  if (s) return s;
  const size_t n = (size_t)d.P * d.V;
  // mean = sum / T, var = (sum2 - T mean^2) / (T - 1)  (mcmc.cpp:877-881)
  std::vector<double> sum(n), sq(n);
  CK(d2h(ctx, sum.data(), c.dev.acc_sum, sizeof(double) * n));
  CK(d2h(ctx, sq.data(), c.dev.acc_sq, sizeof(double) * n));
  const double T = (double)nk;
  for (size_t i = 0; i < n; ++i) {
    const double m = sum[i] / T;
    if (mean) mean[i] = m;
    if (var) var[i] = (sq[i] - T * m * m) / (T - 1.0);
  }
  if (prb && d.S) {
    CK(d2h(ctx, prb, c.dev.prb_sum, sizeof(double) * (size_t)d.S * d.V));
    for (size_t i = 0; i < (size_t)d.S * d.V; ++i) prb[i] /= T;
  }
  if (nkept) *nkept = nk;
  return BSG_OK;
}

bsg_status bsg_get_maps(bsg_ctx *ctx, int32_t chain, double *spatcoef,
                        double *spatcoef_var, double *standcoef, double *prb) {
  if (!valid_chain(ctx, chain)) return BSG_ERR_INVALID;
  const Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  const size_t n = (size_t)d.P * d.V;
  std::vector<double> mean(n), var(n), pr((size_t)d.S * d.V + 1);
  int64_t nk = 0;
  bsg_status s = bsg_get_posterior(ctx, chain, mean.data(), var.data(), pr.data(), &nk);
  if (s) return s;
  const size_t R = (size_t)d.X * d.Y * d.Z;
  const int sy = d.PX, sz = d.PX * d.PY;
  auto grid_of = [&](int v) {
    const int p = d.pad_of_v[v];
    const int k = p / sz, rem = p - k * sz, j = rem / sy, i = rem - j * sy;
    return (size_t)(i - 1) + (size_t)d.X * (j - 1) + (size_t)d.X * d.Y * (k - 1);
  };
  if (spatcoef) std::fill(spatcoef, spatcoef + (size_t)d.P * R, 0.0);
  if (spatcoef_var) std::fill(spatcoef_var, spatcoef_var + (size_t)d.P * R, 0.0);
  if (standcoef) std::fill(standcoef, standcoef + (size_t)d.P * R, 0.0);
  if (prb) std::fill(prb, prb + (size_t)d.S * R, 0.0);
  for (int v = 0; v < d.V; ++v) {
    const size_t r = grid_of(v);
    for (int p = 0; p < d.P; ++p) {
      const double m = mean[(size_t)p * d.V + v], va = var[(size_t)p * d.V + v];
      if (spatcoef) spatcoef[(size_t)p * R + r] = m;
      if (spatcoef_var) spatcoef_var[(size_t)p * R + r] = va;
      if (standcoef && va > 0) standcoef[(size_t)p * R + r] = m / std::sqrt(va);
    }
    if (prb)
      for (int g = 0; g < d.S; ++g) prb[(size_t)g * R + r] = pr[(size_t)g * d.V + v];
  }
  return BSG_OK;
}

bsg_status bsg_reset_accumulators(bsg_ctx *ctx, int32_t chain) {
  if (!valid_chain(ctx, chain)) return BSG_ERR_INVALID;
  const Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  const size_t n = (size_t)d.P * d.V;
  CK(cudaMemsetAsync(c.dev.acc_sum, 0, sizeof(double) * n, ctx->stream));
  CK(cudaMemsetAsync(c.dev.acc_sq, 0, sizeof(double) * n, ctx->stream));
  if (d.S) CK(cudaMemsetAsync(c.dev.prb_sum, 0, sizeof(double) * (size_t)d.S * d.V, ctx->stream));
  CK(cudaMemsetAsync(c.dev.nkept, 0, sizeof(long long), ctx->stream));
  CK(cudaMemsetAsync(c.dev.wm_sum, 0, sizeof(double), ctx->stream));
  if (c.dev.pred_part) {
    CK(cudaMemsetAsync(c.dev.qhat, 0, sizeof(double) * (size_t)d.N * std::max(d.S, 1), ctx->stream));
    CK(cudaMemsetAsync(c.dev.pred_sums, 0, sizeof(double) * 2, ctx->stream));
    CK(cudaMemsetAsync(c.dev.npred, 0, sizeof(long long), ctx->stream));
  }
  return BSG_OK;
}

namespace {
struct CkptHeader {
  uint64_t magic;
  int32_t version, P, Vp, V, S, df_offset, burnin, thin;
  uint32_t key0, key1, chain_id;
  float beta_wm;
};
constexpr uint64_t kCkptMagic = 0x4253474C4D4D4B31ull;  // "BSGLMMK1"

// Version 2 appends the predictive pass: PredCkpt and Qhat [N][max(S,1)].
struct PredCkpt {
  int32_t on, allocated;
  long long npred;
  double ed_sum;
};
struct WmCkpt {  // beta_WM state; the header holds the current value
  int32_t update, pad;
  double sum;
};

size_t ckpt_bytes_v1(const Dataset &d) {
  return sizeof(CkptHeader) + sizeof(float) * (size_t)d.P * d.Vp +
         sizeof(double) * (size_t)d.P * d.P + sizeof(ChainCounters) +
         sizeof(double) * ((size_t)2 * d.P * d.V + (size_t)d.S * d.V);
}

struct MixCkpt {  // link (MODEL); its weights phi follow unless probit
  int32_t model;
  int32_t bits;     // 64: an FP64 chain, whose beta64 [P][Vp] follows (0 = 32)
};

// Version 2 layout: the v1 body, PredCkpt, Qhat [N][max(S,1)], WmCkpt,
// MixCkpt, then phi [N][n_0] and [N][n_1] for the t/logit links, then the
// FP64 coefficients of an FP64 chain.
size_t ckpt_fixed(const Dataset &d) {
  return ckpt_bytes_v1(d) + sizeof(PredCkpt) +
         sizeof(double) * (size_t)d.N * std::max(d.S, 1) + sizeof(WmCkpt) +
         sizeof(MixCkpt);
}

size_t ckpt_bytes(const Dataset &d, int model, bool fp64) {
  return ckpt_fixed(d) +
         (model != 1 ? sizeof(float) * (size_t)d.N * (d.vox[0].size() + d.vox[1].size())
                     : 0) +
         (fp64 ? sizeof(double) * (size_t)d.P * d.Vp : 0);
}
}  // namespace

int64_t bsg_checkpoint_size(const bsg_ctx *ctx, int32_t chain) {
  if (!valid_chain(ctx, chain)) return -1;
  const Chain &c = ctx->ch[chain];
  return (int64_t)ckpt_bytes(ctx->ds[c.dataset], c.dev.model, c.dev.fp64 != 0);
}

bsg_status bsg_checkpoint(bsg_ctx *ctx, int32_t chain, void *buf, int64_t size) {
  if (!valid_chain(ctx, chain) || !buf) return BSG_ERR_INVALID;
  const Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  if (size < (int64_t)ckpt_bytes(d, c.dev.model, c.dev.fp64 != 0))
    return fail(ctx, BSG_ERR_INVALID, "buffer too small");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  char *p = static_cast<char *>(buf);
  WmState ws{};
  CK(d2h(ctx, &ws, c.dev.wm_sum, sizeof(ws)));
  CkptHeader h{kCkptMagic, 2, d.P, d.Vp, d.V, d.S, c.dev.df_offset, c.dev.burnin,
               c.dev.thin, c.dev.key0, c.dev.key1, c.dev.chain_id, ws.beta};
  std::memcpy(p, &h, sizeof(h));
  p += sizeof(h);
  auto get = [&](const void *src, size_t n) -> cudaError_t {
    cudaError_t e = d2h(ctx, p, src, n);
    p += n;
    return e;
  };
  CK(get(c.dev.beta, sizeof(float) * (size_t)d.P * d.Vp));
  CK(get(c.dev.omega_d, sizeof(double) * (size_t)d.P * d.P));
  CK(get(counters_of(c), sizeof(ChainCounters)));
  CK(get(c.dev.acc_sum, sizeof(double) * (size_t)d.P * d.V));
  CK(get(c.dev.acc_sq, sizeof(double) * (size_t)d.P * d.V));
  if (d.S) CK(get(c.dev.prb_sum, sizeof(double) * (size_t)d.S * d.V));
  const size_t nq = (size_t)d.N * std::max(d.S, 1);
  PredCkpt pk{c.pred_on ? 1 : 0, c.dev.pred_part ? 1 : 0, 0, 0.0};
  if (c.dev.pred_part) {
    CK(d2h(ctx, &pk.npred, c.dev.npred, sizeof(long long)));
    CK(d2h(ctx, &pk.ed_sum, c.dev.pred_sums, sizeof(double)));
  }
  std::memcpy(p, &pk, sizeof(pk));
  p += sizeof(pk);
  if (c.dev.pred_part)
    CK(get(c.dev.qhat, sizeof(double) * nq));
  else {
    std::memset(p, 0, sizeof(double) * nq);
    p += sizeof(double) * nq;
  }
  const WmCkpt wk{c.dev.wm_update, 0, ws.sum};
  std::memcpy(p, &wk, sizeof(wk));
  p += sizeof(wk);
  const MixCkpt mk{c.dev.model, c.dev.fp64 ? 64 : 0};
  std::memcpy(p, &mk, sizeof(mk));
  p += sizeof(mk);
  if (c.dev.model != 1)
    for (int k = 0; k < 2; ++k)
      CK(get(c.dev.phi[k], sizeof(float) * (size_t)d.N * d.vox[k].size()));
  if (c.dev.fp64) CK(get(c.dev.beta64, sizeof(double) * (size_t)d.P * d.Vp));
  return BSG_OK;
}

bsg_status bsg_restore(bsg_ctx *ctx, int32_t chain, const void *buf, int64_t size) {
  if (!valid_chain(ctx, chain) || !buf) return BSG_ERR_INVALID;
  Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  CkptHeader h;
  if (size < (int64_t)sizeof(h)) return fail(ctx, BSG_ERR_INVALID, "not a checkpoint");
  std::memcpy(&h, buf, sizeof(h));
  if (h.magic != kCkptMagic || (h.version != 1 && h.version != 2))
    return fail(ctx, BSG_ERR_INVALID, "not a checkpoint");
  if (h.P != d.P || h.Vp != d.Vp || h.V != d.V || h.S != d.S ||
      size < (int64_t)(h.version == 1 ? ckpt_bytes_v1(d) : ckpt_fixed(d)))
    return fail(ctx, BSG_ERR_INVALID, "checkpoint is for a study of another shape");
  MixCkpt mk{1, 0};
  if (h.version == 2) {
    std::memcpy(&mk, static_cast<const char *>(buf) + ckpt_fixed(d) - sizeof(MixCkpt),
                sizeof(mk));
    if (mk.model < 0 || mk.model > 2 || (mk.bits != 0 && mk.bits != 64) ||
        (mk.bits == 64 && mk.model != 1) ||
        size < (int64_t)ckpt_bytes(d, mk.model, mk.bits == 64))
      return fail(ctx, BSG_ERR_INVALID, "checkpoint is for a study of another shape");
  }
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  const char *p = static_cast<const char *>(buf) + sizeof(h);
  auto put = [&](void *dst, size_t n) -> cudaError_t {
    cudaError_t e = h2d(ctx, dst, p, n);
    p += n;
    return e;
  };
  CK(put(c.dev.beta, sizeof(float) * (size_t)d.P * d.Vp));
  std::vector<double> om((size_t)d.P * d.P);
  std::memcpy(om.data(), p, sizeof(double) * om.size());
  CK(put(c.dev.omega_d, sizeof(double) * om.size()));
  std::vector<float> omf(om.begin(), om.end());
  CK(h2d(ctx, c.dev.omega_f, omf.data(), sizeof(float) * omf.size()));
  CK(put(counters_of(c), sizeof(ChainCounters)));
  CK(put(c.dev.acc_sum, sizeof(double) * (size_t)d.P * d.V));
  CK(put(c.dev.acc_sq, sizeof(double) * (size_t)d.P * d.V));
  if (d.S) CK(put(c.dev.prb_sum, sizeof(double) * (size_t)d.S * d.V));
  PredCkpt pk{0, 0, 0, 0.0};
  if (h.version == 2) {
    std::memcpy(&pk, p, sizeof(pk));
    p += sizeof(pk);
  }
  const size_t nq = (size_t)d.N * std::max(d.S, 1);
  if (pk.allocated || c.dev.pred_part) {
    bsg_status ps = ensure_pred(ctx, c);
    if (ps) return ps;
    if (pk.allocated)
      CK(h2d(ctx, c.dev.qhat, p, sizeof(double) * nq));
    else
      CK(cudaMemsetAsync(c.dev.qhat, 0, sizeof(double) * nq, ctx->stream));
    CK(h2d(ctx, c.dev.npred, &pk.npred, sizeof(long long)));
    const double sums[2] = {pk.ed_sum, 0.0};
    CK(h2d(ctx, c.dev.pred_sums, sums, sizeof(sums)));
  }
  if (h.version == 2) p += sizeof(double) * nq;
  c.pred_on = pk.on != 0;
  WmCkpt wk{0, 0, 0.0};
  if (h.version == 2) {
    std::memcpy(&wk, p, sizeof(wk));
    p += sizeof(wk) + sizeof(MixCkpt);
  } else {
    long long nk = 0;  // v1: beta_WM was fixed, so its kept sum is nk beta_WM
    CK(d2h(ctx, &nk, c.dev.nkept, sizeof(nk)));
    wk.sum = (double)nk * (double)h.beta_wm;
  }
  if (wk.update && !d.dev.has_c)
    return fail(ctx, BSG_ERR_UNSUPPORTED, "checkpoint has the beta_WM update on");
  const WmState ws{wk.sum, h.beta_wm, 0};
  CK(h2d(ctx, c.dev.wm_sum, &ws, sizeof(ws)));
  c.dev.wm_update = wk.update;
  if (mk.model != c.dev.model) {
    bsg_status ms = set_model(ctx, c, mk.model);
    if (ms) return ms;
  }
  if (mk.model != 1)
    for (int k = 0; k < 2; ++k)
      CK(put(c.dev.phi[k], sizeof(float) * (size_t)d.N * d.vox[k].size()));
  {
    bsg_status fs = set_precision(ctx, c, mk.bits == 64 ? 64 : 32);
    if (fs) return fs;
  }
  if (mk.bits == 64) CK(put(c.dev.beta64, sizeof(double) * (size_t)d.P * d.Vp));
  c.desc.beta_wm = h.beta_wm;
  c.dev.df_offset = h.df_offset;
  c.dev.burnin = h.burnin;
  c.dev.thin = h.thin;
  c.dev.key0 = h.key0;
  c.dev.key1 = h.key1;
  c.dev.chain_id = h.chain_id;
  ctx->plan_valid = false;  // descriptors changed
  return BSG_OK;
}

bsg_status bsg_autotune(bsg_ctx *ctx, int32_t sweeps, int32_t *best_lpv,
                        int32_t *best_threads) {
  if (!ctx || sweeps < 1) return BSG_ERR_INVALID;
  if (ctx->ch.empty()) return fail(ctx, BSG_ERR_STATE, "no chain");
  std::vector<std::vector<char>> saved(ctx->ch.size());
  for (size_t i = 0; i < ctx->ch.size(); ++i) {
    saved[i].resize(ckpt_bytes(ctx->ds[ctx->ch[i].dataset], ctx->ch[i].dev.model,
                               ctx->ch[i].dev.fp64 != 0));
    bsg_status s = bsg_checkpoint(ctx, (int32_t)i, saved[i].data(), (int64_t)saved[i].size());
    if (s) return s;
  }
  const int lpvs[] = {1, 2, 4, 8}, thrs[] = {64, 128, 256};
  double best = 1e300;
  int bl = ctx->lpv, bt = ctx->threads, bstep = ctx->step;
  bool btc = ctx->tc;
  for (int lpv : lpvs)
    for (int thr : thrs)
      for (int tc = 0; tc < (lpv == 1 ? 2 : 1); ++tc)  // X'Z: SIMT, tensor cores
        for (int step : {0, 16, 8}) {  // subjects per step: per group, 16, 8
          if (step && (lpv != 1 || tc)) continue;  // those take the 8-subject step
          if (thr / lpv < 8) continue;
          bsg_status s = bsg_set_tuning(ctx, lpv, thr);
          if (!s) s = bsg_set_tensor_xz(ctx, tc);
          if (!s) s = bsg_set_step_subjects(ctx, step);
          if (!s) s = bsg_run(ctx, 1);  // warm-up and graph capture
          double ms = 0;
          if (!s) s = bsg_run_timed(ctx, sweeps, &ms);
          for (size_t i = 0; i < ctx->ch.size() && !s; ++i)
            s = bsg_restore(ctx, (int32_t)i, saved[i].data(), (int64_t)saved[i].size());
          if (s) return s;
          if (ms < best) {
            best = ms;
            bl = lpv;
            bt = thr;
            btc = tc != 0;
            bstep = step;
          }
        }
  bsg_status s = bsg_set_tuning(ctx, bl, bt);
  if (!s) s = bsg_set_tensor_xz(ctx, btc ? 1 : 0);
  if (!s) s = bsg_set_step_subjects(ctx, bstep);
  if (s) return s;
  if (best_lpv) *best_lpv = bl;
  if (best_threads) *best_threads = bt;
  return BSG_OK;
}

bsg_status bsg_sweep_supplied(bsg_ctx *ctx, int32_t chain, const uint32_t *ubits,
                              const float *normals, const double *chi2,
                              const double *wnorm, int32_t form) {
  if (!valid_chain(ctx, chain) || !ubits || !normals || !chi2 || !wnorm)
    return BSG_ERR_INVALID;
  if (form != 0 && form != 1) return fail(ctx, BSG_ERR_INVALID, "form must be 0 or 1");
  CK(cudaSetDevice(ctx->device));
  bsg_status s = build_plan(ctx);
  if (s) return s;
  const Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  if (c.dev.wm_update)
    return fail(ctx, BSG_ERR_UNSUPPORTED,
                "supplied-variate sweeps take beta_WM as given (turn its update off)");
  if (c.dev.model != 1)
    return fail(ctx, BSG_ERR_UNSUPPORTED, "supplied-variate sweeps are probit only");
  if (c.dev.fp64)
    return fail(ctx, BSG_ERR_UNSUPPORTED, "supplied-variate sweeps run in FP32");
  cudaError_t e;
  const int P = d.P, nw = P * (P - 1) / 2;
  Supplied sup{};
  uint32_t *du = upload(ctx, ubits, (size_t)d.N * d.V, &e);
  CK(e);
  float *dn = upload(ctx, normals, (size_t)d.V * P, &e);
  CK(e);
  double *dc = upload(ctx, chi2, (size_t)P, &e);
  CK(e);
  double *dw = upload(ctx, wnorm, (size_t)(nw ? nw : 1), &e);
  CK(e);
  sup.ubits = du;
  sup.normals = dn;
  sup.chi2 = dc;
  sup.wnorm = dw;
  sup.form = form;
  // Block maps for this chain alone, one lane per voxel.
  const int thr = kParityThreads;
  std::vector<BlockMap> m[2];
  for (int col = 0; col < 2; ++col) map_chain(m[col], chain, (int)d.vox[col].size(), thr, col);
  e = cudaSuccess;
  BlockMap *dm0 = m[0].empty() ? nullptr : upload(ctx, m[0].data(), m[0].size(), &e);
  CK(e);
  BlockMap *dm1 = upload(ctx, m[1].data(), m[1].size(), &e);
  CK(e);
  CK(launch_fused(P, 1, thr, true, ctx->d_ds, ctx->d_ch, dm0, (int)m[0].size(), 0, sup,
                  ctx->stream));
  CK(launch_fused(P, 1, thr, true, ctx->d_ds, ctx->d_ch, dm1, (int)m[1].size(), 1, sup,
                  ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (void *p : {(void *)du, (void *)dn, (void *)dc, (void *)dw, (void *)dm0,
                  (void *)dm1})
    dfree(ctx, p);
  return bsg_sync(ctx);
}

// ------------------------------------------------------------ the link --
bsg_status bsg_set_model(bsg_ctx *ctx, int32_t chain, int32_t model) {
  if (!valid_chain(ctx, chain) || model < 0 || model > 2) return BSG_ERR_INVALID;
  Chain &c = ctx->ch[chain];
  if (model != 1 && c.dev.wm_update)
    return fail(ctx, BSG_ERR_UNSUPPORTED, "the beta_WM update is probit only");
  if (model != 1 && c.dev.fp64)
    return fail(ctx, BSG_ERR_UNSUPPORTED, "FP64 chains are probit only");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  return set_model(ctx, c, model);
}

// ------------------------------------------------------- FP64 chains ----
bsg_status bsg_set_precision(bsg_ctx *ctx, int32_t chain, int32_t bits) {
  if (!valid_chain(ctx, chain) || (bits != 32 && bits != 64)) return BSG_ERR_INVALID;
  Chain &c = ctx->ch[chain];
  if (bits == 64 && c.dev.model != 1)
    return fail(ctx, BSG_ERR_UNSUPPORTED, "FP64 chains are probit only");
  if (bits == 64 && c.dev.wm_update)
    return fail(ctx, BSG_ERR_UNSUPPORTED, "FP64 chains keep beta_WM fixed");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  return set_precision(ctx, c, bits);
}

bsg_status bsg_get_beta64(bsg_ctx *ctx, int32_t chain, double *out) {
  if (!valid_chain(ctx, chain) || !out) return BSG_ERR_INVALID;
  const Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  const size_t n = (size_t)d.P * d.Vp;
  CK(cudaSetDevice(ctx->device));
  if (c.dev.fp64) {
    CK(d2h(ctx, out, c.dev.beta64, sizeof(double) * n));
  } else {
    std::vector<float> bf(n);
    CK(d2h(ctx, bf.data(), c.dev.beta, sizeof(float) * n));
    std::copy(bf.begin(), bf.end(), out);
  }
  return BSG_OK;
}

// ------------------------------------------------ DIC / Qhat predictive --
bsg_status bsg_set_predictive(bsg_ctx *ctx, int32_t chain, int32_t enable) {
  if (!valid_chain(ctx, chain)) return BSG_ERR_INVALID;
  Chain &c = ctx->ch[chain];
  if (ctx->ds[c.dataset].S < 1)
    return fail(ctx, BSG_ERR_INVALID, "the predictive pass needs a group column (S >= 1)");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  if (enable) {
    bsg_status s = ensure_pred(ctx, c);
    if (s) return s;
  }
  if (c.pred_on != (enable != 0)) ctx->plan_valid = false;
  c.pred_on = enable != 0;
  return BSG_OK;
}

bsg_status bsg_predict(bsg_ctx *ctx, int32_t chain, double *mpredict) {
  if (!valid_chain(ctx, chain) || !mpredict) return BSG_ERR_INVALID;
  Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  if (d.S < 1)
    return fail(ctx, BSG_ERR_INVALID, "the predictive pass needs a group column (S >= 1)");
  CK(cudaSetDevice(ctx->device));
  bsg_status s = ensure_pred(ctx, c);
  if (s) return s;
  if ((s = build_plan(ctx))) return s;
  const int chunks = (d.N + kPredThreads - 1) / kPredThreads;
  CK(launch_predict(d.P, d.S, ctx->d_ds, ctx->d_ch, nullptr, c.dev.pred_tiles, chunks,
                    chain, kPredNow, ctx->stream, false));
  CK(launch_predict_finish(ctx->d_ds, ctx->d_ch, nullptr,
                           (d.N + kPredWarps - 1) / kPredWarps, chain, kPredNow,
                           ctx->stream, false));
  CK(d2h(ctx, mpredict, c.dev.mpred, sizeof(double) * (size_t)d.N * d.S));
  return BSG_OK;
}

bsg_status bsg_get_predictive(bsg_ctx *ctx, int32_t chain, double *qhat,
                              double *ed_sum, int64_t *npred) {
  if (!valid_chain(ctx, chain)) return BSG_ERR_INVALID;
  const Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  const size_t nq = (size_t)d.N * d.S;
  long long n = 0;
  double ed = 0.0;
  if (c.dev.pred_part) {
    CK(d2h(ctx, &n, c.dev.npred, sizeof(n)));
    CK(d2h(ctx, &ed, c.dev.pred_sums, sizeof(ed)));
    if (qhat && nq) CK(d2h(ctx, qhat, c.dev.qhat, sizeof(double) * nq));
  } else if (qhat && nq) {
    std::memset(qhat, 0, sizeof(double) * nq);
  }
  if (ed_sum) *ed_sum = ed;
  if (npred) *npred = n;
  return BSG_OK;
}

bsg_status bsg_get_dic(bsg_ctx *ctx, int32_t chain, double *dic) {
  if (!valid_chain(ctx, chain) || !dic) return BSG_ERR_INVALID;
  Chain &c = ctx->ch[chain];
  const Dataset &d = ctx->ds[c.dataset];
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  long long nk = 0, np = 0;
  CK(d2h(ctx, &nk, c.dev.nkept, sizeof(nk)));
  if (c.dev.pred_part) CK(d2h(ctx, &np, c.dev.npred, sizeof(np)));
  if (nk < 1 || np < 1)
    return fail(ctx, BSG_ERR_STATE,
                "DIC needs kept sweeps with the predictive pass on (bsg_set_predictive)");
  bsg_status s = build_plan(ctx);
  if (s) return s;
  const int chunks = (d.N + kPredThreads - 1) / kPredThreads;
  CK(launch_predict(d.P, d.S, ctx->d_ds, ctx->d_ch, nullptr, c.dev.pred_tiles, chunks,
                    chain, kPredDE, ctx->stream, false));
  CK(launch_predict_finish(ctx->d_ds, ctx->d_ch, nullptr,
                           (d.N + kPredWarps - 1) / kPredWarps, chain, kPredDE,
                           ctx->stream, false));
  CK(cudaStreamSynchronize(ctx->stream));
  double sums[2];
  CK(d2h(ctx, sums, c.dev.pred_sums, sizeof(sums)));
  // mcmc.cpp:966-975
  const double DE = sums[1];
  const double ED = -2.0 * sums[0] / (double)np;
  const double PD = ED - DE;
  dic[0] = DE;
  dic[1] = ED;
  dic[2] = PD;
  dic[3] = DE + 2.0 * PD;
  return BSG_OK;
}

}  // extern "C"
