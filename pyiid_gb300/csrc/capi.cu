// capi.cu -- context, host-side layouts and the C ABI of include/pyiid_gb300.h.
//
// Host responsibilities (all O(N) or O(K*R), cached by content hash):
//   * Layout: per configuration, a stable species sort (perm), tiles of at
//     most 32 atoms that never straddle a (configuration, species) boundary,
//     the F(Q) work items (tile I, run of tiles J <= I of one species) grouped
//     by (configuration, species pair), and the pair counts per species pair.
//   * na(Q): n * mean_{a>b} f_a f_b per configuration in FP64.
//   * T: the linear map equal to the reference's F -> G FFT transform.
// Device work is enqueued on the context stream; device buffers only grow.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/pyiid_gb300.h"
#include "debye_kernels.cuh"
#include "move_kernels.cuh"
#include "spring_kernels.cuh"
#include "transform_kernels.cuh"
#include "umma_gemm.cuh"

using namespace pyiid;

namespace {

constexpr int kVersion = 10000;  // 1.0.0
constexpr int kJMax = kJMaxTiles;  // max J tiles per F(Q) work item
constexpr int kAdjRS = 128;      // adjoint re-seed period (bins)

// ---------------------------------------------------------------- variants
// Launch shapes of the two pair kernels; pyiid_tune selects one per context.
// F(Q): L bins per thread, NP pairs interleaved per thread.
struct FqVariant {
  int L, NP;
};
// dF/dx: L bins per thread, CPC chunks (threads) per atom in a CTA, NP pairs.
struct GradVariant {
  int L, CPC, NP;
};

using FqKernel = void (*)(const float *, const int *, const int4 *,
                          const int4 *, const int *, float, float, int, int,
                          int, int, double *);
using GradKernel = void (*)(const float *, const int *, const int4 *,
                            const int2 *, float, float, int, int, int,
                            const float *, int, float *, JSplit);

using FqPersistKernel = void (*)(const float *, const int *, const int4 *,
                                 const int4 *, const int *, float, float, int,
                                 int, int, int, int, int, int *, double *);
struct FqEntry {
  FqVariant v;
  FqKernel k;             // one CTA per work unit
  FqPersistKernel kp = nullptr;  // persistent form of the same shape
};
struct GradEntry {
  GradVariant v;
  GradKernel k;
};
using FqGradKernel = void (*)(const float *, const int *, const int4 *,
                              const int2 *, float, float, int, int, int,
                              const float *, int, float *, const float *,
                              double *, int, JSplit);
struct FqGradEntry {
  GradVariant v;
  FqGradKernel k;
};

// NP <= 0 marks the packed (FP32x2) even/odd kernels: 0 one pair per
// thread at a time, -2 two pairs interleaved, -3 (and -4) the per-tile-pair
// group reduction at 3 (4) CTAs per SM, -13 its persistent form (CTAs
// resident on every SM taking work units from a counter) at 3 CTAs per SM
const FqEntry kFqTable[] = {
    {{32, 0}, fq_pair2_kernel<32>},   {{48, 0}, fq_pair2_kernel<48>},
    {{64, 0}, fq_pair2_kernel<64>},   {{24, 0}, fq_pair2_kernel<24>},
    {{32, -2}, fq_pair2_kernel<32, 2>},
    {{48, -2}, fq_pair2_kernel<48, 2>},
    {{24, -2}, fq_pair2_kernel<24, 2>},
    {{16, -2}, fq_pair2_kernel<16, 2>},
    {{32, 1}, fq_pair_kernel<32, 1>}, {{32, 2}, fq_pair_kernel<32, 2>},
    {{16, 1}, fq_pair_kernel<16, 1>}, {{16, 2}, fq_pair_kernel<16, 2>},
    {{24, 1}, fq_pair_kernel<24, 1>}, {{24, 2}, fq_pair_kernel<24, 2>},
    {{48, 1}, fq_pair_kernel<48, 1>}, {{16, 4}, fq_pair_kernel<16, 4>},
    {{32, -3}, fq_pair3_kernel<32, 3>}, {{32, -4}, fq_pair3_kernel<32, 4>},
    {{24, -3}, fq_pair3_kernel<24, 3>}, {{24, -4}, fq_pair3_kernel<24, 4>},
    {{16, -4}, fq_pair3_kernel<16, 4>},
    {{48, -3}, fq_pair3_kernel<48, 3>}, {{40, -3}, fq_pair3_kernel<40, 3>},
    {{56, -3}, fq_pair3_kernel<56, 3>},
    {{56, -13}, fq_pair3_kernel<56, 3>, fq_pair3_persistent<56, 3>},
    {{48, -13}, fq_pair3_kernel<48, 3>, fq_pair3_persistent<48, 3>},
    {{40, -13}, fq_pair3_kernel<40, 3>, fq_pair3_persistent<40, 3>},
};
// (the last template argument is the minimum resident CTAs per SM, i.e. the
// register budget: 2 x 256 threads -> 128 registers, 3 x 256 -> 85)
const GradEntry kGradTable[] = {
    {{32, 8, 0}, gradfq2_kernel<32, 8, 2>},
    {{24, 8, 0}, gradfq2_kernel<24, 8, 2>},
    {{16, 8, 0}, gradfq2_kernel<16, 8, 3>},
    {{32, 16, 0}, gradfq2_kernel<32, 16, 1>},
    {{32, 8, 1}, gradfq_kernel<32, 8, 1, 2>},
    {{32, 16, 1}, gradfq_kernel<32, 16, 1, 1>},
    {{32, 4, 1}, gradfq_kernel<32, 4, 1, 4>},
    {{16, 8, 1}, gradfq_kernel<16, 8, 1, 3>},
    {{16, 8, 2}, gradfq_kernel<16, 8, 2, 2>},
    {{16, 16, 2}, gradfq_kernel<16, 16, 2, 1>},
    {{24, 8, 1}, gradfq_kernel<24, 8, 1, 2>},
    {{16, 4, 1}, gradfq_kernel<16, 4, 1, 6>},
};
// F(Q) + dF/dx in one pass (packed kernels only)
const FqGradEntry kFqGradTable[] = {
    {{24, 8, 0}, fqgrad2_kernel<24, 8, 2>},
    {{32, 8, 0}, fqgrad2_kernel<32, 8, 1>},
    {{16, 8, 0}, fqgrad2_kernel<16, 8, 2>},
    {{32, 16, 0}, fqgrad2_kernel<32, 16, 1>},
    {{24, 16, 0}, fqgrad2_kernel<24, 16, 1>},
};
constexpr int kNumFqGrad = sizeof(kFqGradTable) / sizeof(kFqGradTable[0]);
// dF/dx alone: the packed kernels keep four record arrays per tile pair
// (the fourth: pair-only products), the scalar ones three
size_t grad_smem(const GradVariant &v) {
  return (v.NP == 0 ? 4 : 3) * kTile * kTile * sizeof(float4);
}
size_t fqgrad_smem(const GradVariant &v) {
  return 4 * kTile * kTile * sizeof(float4) +
         (2 * (size_t)v.CPC * v.CPC * v.L + kTile * kTile) * sizeof(float);
}
constexpr int kNumFq = sizeof(kFqTable) / sizeof(kFqTable[0]);
// Default F(Q) launch shape of a new context: {56, -3}, the per-tile-pair
// group reduction with 56 bins per thread at 3 CTAs per SM.  The tuner
// picks it on 330, 498 and 500-bin workloads (64 x 1,000 atoms, 256
// alloys, one 1,000-atom particle) and it is within 1 % of the fastest at
// 1,475 bins and 20,000 atoms; the autotuner may pick another.
constexpr int kDefaultFq = 23;
constexpr int kNumGrad = sizeof(kGradTable) / sizeof(kGradTable[0]);

// Dynamic shared memory of an F(Q) launch with n_chunks chunks per CTA
// (n_chunks < 0: the upper bound over all launches, for the attribute).
size_t fq_smem(const FqVariant &v, int n_chunks = -1) {
  if (v.NP <= -3) {  // records / group scratch + FP64 per-bin accumulators
    const size_t acc = n_chunks < 0 ? 32768 : (size_t)n_chunks * v.L * 8;
    return (size_t)fq3_scratch_floats(v.L) * sizeof(float) + acc;
  }
  return 2 * kTile * kTile * sizeof(float4) +
         2 * (size_t)v.L * kBlock * sizeof(float);
}

// Cache key of host arrays (r grids, species, form-factor tables) that are
// hashed on every call: eight bytes per step (an FNV-style multiply followed
// by an xor-shift so that high bits reach the low ones), then the tail byte
// by byte.  A 4,000-point r grid takes a few microseconds.
uint64_t fnv1a(const void *data, size_t n, uint64_t h = 1469598103934665603ull) {
  const unsigned char *p = static_cast<const unsigned char *>(data);
  size_t i = 0;
  for (; i + 8 <= n; i += 8) {
    uint64_t w;
    std::memcpy(&w, p + i, 8);
    h = (h ^ w) * 1099511628211ull;
    h ^= h >> 29;
  }
  for (; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}
template <class T>
uint64_t mix(uint64_t h, const T &v) {
  return fnv1a(&v, sizeof(T), h);
}

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

struct Layout {
  uint64_t key = 0;
  int total = 0, n_configs = 0, n_species = 0, n_spairs = 0;
  std::vector<int> offsets, perm;
  std::vector<int4> tiles;
  std::vector<int2> cfg_tiles;
  std::vector<int4> items;
  std::vector<int> item_order;  // launch order: items by decreasing pairs
  std::vector<int> key_item_begin;
  std::vector<int2> spair_species;
  std::vector<double> pair_counts;  // [n_configs][n_spairs]
  std::vector<int> natoms;          // per configuration
  // symmetric adjoint: per item the float offsets of its i-side [32][3] and
  // j-side [(J1-J0)*32][3] partial rows; per tile the CSR list of the
  // [32][3] blocks that sum to its gradient rows
  std::vector<int> adj_ioff, adj_joff, adj_tile_ptr, adj_entries;
  size_t adj_total = 0;
  // single-atom moves: items (configuration, species, tile run [t0, t1)) of
  // at most kMoveTiles tiles, CSR by configuration
  std::vector<int4> mitems;
  std::vector<int> mitem_begin;
  int4 *d_mitems = nullptr;
  int *d_mitem_begin = nullptr;
  int *d_offsets = nullptr;
  int *d_species = nullptr;
  int *d_adj_ioff = nullptr;
  int *d_adj_joff = nullptr;
  int *d_adj_tile_ptr = nullptr;
  int *d_adj_entries = nullptr;
  // device copies
  int *d_perm = nullptr;
  int4 *d_tiles = nullptr;
  int2 *d_cfg_tiles = nullptr;
  int4 *d_items = nullptr;
  int *d_item_order = nullptr;
  int *d_key_item_begin = nullptr;
  int2 *d_spair = nullptr;
};

struct TMatrix {
  uint64_t key = 0;
  int n_bins = 0, n_r = 0, kmin = 0;
  float *d_T = nullptr;
  // Gram matrix T T^T (single-atom moves), built on first use
  double *d_M64 = nullptr;
  float *d_M32 = nullptr;
  // T^T scaled by 2^e_t and split into FP16 high and low parts, packed for
  // the tensor-core G(r) gradient (umma::pack_b_f16_kernel), built on first
  // use; t_amax = max |T| over the bins from kmin
  void *d_Bhi = nullptr, *d_Blo = nullptr;
  int b_rows_pad = 0, e_t = 0;
  float t_amax = 0.f;
};

void free_tmatrix(TMatrix *M) {
  cudaFree(M->d_T);
  cudaFree(M->d_M64);
  cudaFree(M->d_M32);
  cudaFree(M->d_Bhi);
  cudaFree(M->d_Blo);
}

struct NaTable {
  uint64_t key = 0;
  double *d_na = nullptr;
};

std::mutex g_err_mu;
std::string g_err;  // errors without a context

}  // namespace

struct pyiid_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int64_t launches = 0;
  std::unordered_map<std::string, DevBuf> bufs;
  std::vector<std::unique_ptr<Layout>> layouts;  // small LRU (front = newest)
  std::vector<std::unique_ptr<TMatrix>> tmats;
  std::vector<std::unique_ptr<NaTable>> nas;
  uint64_t ftab_key = 0;
  int ftab_species = 0, ftab_bins = 0;
  bool attrs_set = false;
  int fq_variant = kDefaultFq;
  int grad_variant = 0;
  int adj_variant = 0;  // 0: symmetric (each pair once), 1: owner-computes
  int fqgrad_variant = 0;
  // 0: mma.sync (mlp_fused_kernel), 1: tcgen05 one tile per CTA, 2: tcgen05
  // two tiles in flight per CTA (default: 57 against 70 us for mma.sync)
  int mlp_variant = 2;
  int n_sms = 0;  // streaming multiprocessors of the device
  // device word a kernel sets when one of its bounded waits gave up
  // (reported and cleared by pyiid_synchronize)
  int *d_status = nullptr;
  // resident CTAs per SM of a persistent kernel at a shared-memory size
  std::map<std::pair<const void *, size_t>, int> occupancy;
};

namespace {

int fail(pyiid_ctx *ctx, int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) {
    ctx->err = buf;
  } else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_err = buf;
  }
  return code;
}

#define CUDA_TRY(ctx, expr)                                                   \
  do {                                                                        \
    cudaError_t e_ = (expr);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? PYIID_ERR_OOM        \
                                                       : PYIID_ERR_CUDA,      \
                  "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_),     \
                  __FILE__, __LINE__);                                        \
    }                                                                         \
  } while (0)

#define LAUNCH_CHECK(ctx)                                                     \
  do {                                                                        \
    ++(ctx)->launches;                                                        \
    cudaError_t e_ = cudaGetLastError();                                      \
    if (e_ != cudaSuccess)                                                    \
      return fail(ctx, PYIID_ERR_CUDA, "kernel launch failed: %s (%s:%d)",    \
                  cudaGetErrorString(e_), __FILE__, __LINE__);                \
  } while (0)

#define TRY(expr)              \
  do {                         \
    int rc_ = (expr);          \
    if (rc_ != PYIID_OK) return rc_; \
  } while (0)

// Grow-only device buffer by name.
int ensure(pyiid_ctx *ctx, const char *name, size_t bytes, void **out) {
  DevBuf &b = ctx->bufs[name];
  if (b.bytes < bytes) {
    if (b.p) CUDA_TRY(ctx, cudaFree(b.p));
    b.p = nullptr;
    b.bytes = 0;
    size_t alloc = std::max<size_t>(bytes, 256);
    CUDA_TRY(ctx, cudaMalloc(&b.p, alloc));
    b.bytes = alloc;
  }
  *out = b.p;
  return PYIID_OK;
}

template <class T>
int upload(pyiid_ctx *ctx, T **dst, const std::vector<T> &src) {
  if (*dst) CUDA_TRY(ctx, cudaFree(*dst));
  *dst = nullptr;
  size_t n = std::max<size_t>(src.size(), 1);
  CUDA_TRY(ctx, cudaMalloc((void **)dst, n * sizeof(T)));
  if (!src.empty())
    CUDA_TRY(ctx, cudaMemcpy(*dst, src.data(), src.size() * sizeof(T),
                             cudaMemcpyHostToDevice));
  return PYIID_OK;
}

void free_layout(Layout *L) {
  cudaFree(L->d_perm);
  cudaFree(L->d_tiles);
  cudaFree(L->d_cfg_tiles);
  cudaFree(L->d_items);
  cudaFree(L->d_item_order);
  cudaFree(L->d_key_item_begin);
  cudaFree(L->d_spair);
  cudaFree(L->d_adj_ioff);
  cudaFree(L->d_adj_joff);
  cudaFree(L->d_adj_tile_ptr);
  cudaFree(L->d_adj_entries);
  cudaFree(L->d_mitems);
  cudaFree(L->d_mitem_begin);
  cudaFree(L->d_offsets);
  cudaFree(L->d_species);
}

// Builds (or finds) the layout of a packed batch.
int get_layout(pyiid_ctx *ctx, const int32_t *species, const int32_t *offsets,
               int n_configs, int n_species, Layout **out) {
  const int total = offsets[n_configs];
  uint64_t key = fnv1a(offsets, sizeof(int32_t) * (n_configs + 1));
  key = fnv1a(species, sizeof(int32_t) * (size_t)total, key);
  key = mix(key, n_species);
  for (size_t i = 0; i < ctx->layouts.size(); ++i) {
    if (ctx->layouts[i]->key == key) {
      if (i != 0) std::swap(ctx->layouts[0], ctx->layouts[i]);
      *out = ctx->layouts[0].get();
      return PYIID_OK;
    }
  }
  for (int i = 0; i < total; ++i)
    if (species[i] < 0 || species[i] >= n_species)
      return fail(ctx, PYIID_ERR_INVALID_ARG,
                  "species[%d] = %d outside [0, %d)", i, species[i], n_species);
  auto L = std::make_unique<Layout>();
  L->key = key;
  L->total = total;
  L->n_configs = n_configs;
  L->n_species = n_species;
  L->n_spairs = n_species * (n_species + 1) / 2;
  L->offsets.assign(offsets, offsets + n_configs + 1);
  L->perm.resize(total);
  L->cfg_tiles.resize(n_configs);
  L->natoms.resize(n_configs);
  L->pair_counts.assign((size_t)n_configs * L->n_spairs, 0.0);
  for (int sa = 0; sa < n_species; ++sa)
    for (int sb = 0; sb <= sa; ++sb) L->spair_species.push_back(make_int2(sa, sb));
  std::vector<int> count(n_species);
  for (int c = 0; c < n_configs; ++c) {
    const int o0 = offsets[c], o1 = offsets[c + 1];
    L->natoms[c] = o1 - o0;
    std::fill(count.begin(), count.end(), 0);
    for (int i = o0; i < o1; ++i) count[species[i]]++;
    std::vector<int> start(n_species, o0);
    for (int s = 1; s < n_species; ++s) start[s] = start[s - 1] + count[s - 1];
    std::vector<int> fillp = start;
    for (int i = o0; i < o1; ++i) L->perm[fillp[species[i]]++] = i;
    const int t0 = (int)L->tiles.size();
    for (int s = 0; s < n_species; ++s)
      for (int a = 0; a < count[s]; a += kTile)
        L->tiles.push_back(
            make_int4(start[s] + a, std::min(kTile, count[s] - a), c, s));
    const int t1 = (int)L->tiles.size();
    L->cfg_tiles[c] = make_int2(t0, t1);
    L->mitem_begin.push_back((int)L->mitems.size());
    for (int t = t0; t < t1;) {
      int te = t;
      while (te < t1 && L->tiles[te].w == L->tiles[t].w && te - t < kMoveTiles)
        ++te;
      L->mitems.push_back(make_int4(c, L->tiles[t].w, t, te));
      t = te;
    }
    for (int sa = 0; sa < n_species; ++sa)
      for (int sb = 0; sb <= sa; ++sb) {
        const double na = count[sa], nb = count[sb];
        L->pair_counts[(size_t)c * L->n_spairs + sa * (sa + 1) / 2 + sb] =
            (sa == sb) ? na * (na - 1) / 2 : na * nb;
      }
  }
  // F(Q) items: tile I with runs of at most jmax tiles J <= I of one
  // species.  Runs are kJMax tiles long unless that leaves fewer than about
  // four items per SM (small batches: one 1,000-atom particle has 32
  // tiles), then shorter, so that the pair kernels still fill the GPU.
  {
    double tile_pairs = 0.0;
    for (int c = 0; c < n_configs; ++c) {
      const double T = L->cfg_tiles[c].y - L->cfg_tiles[c].x;
      tile_pairs += T * (T + 1) / 2;
    }
    const double target = 4.0 * std::max(1, ctx->n_sms);
    const int jmax =
        std::max(1, std::min(kJMax, (int)std::floor(tile_pairs / target)));
    for (int c = 0; c < n_configs; ++c) {
      const int t0 = L->cfg_tiles[c].x, t1 = L->cfg_tiles[c].y;
      for (int I = t0; I < t1; ++I) {
        int J = t0;
        while (J <= I) {
          const int sJ = L->tiles[J].w;
          int Je = J;
          while (Je <= I && L->tiles[Je].w == sJ && Je - J < jmax) ++Je;
          const int sI = L->tiles[I].w;
          const int sp = sI * (sI + 1) / 2 + sJ;
          L->items.push_back(make_int4(I, J, Je, c * L->n_spairs + sp));
          J = Je;
        }
      }
    }
  }
  std::stable_sort(L->items.begin(), L->items.end(),
                   [](const int4 &a, const int4 &b) { return a.w < b.w; });
  const int nkeys = n_configs * L->n_spairs;
  L->key_item_begin.assign(nkeys + 1, 0);
  for (const int4 &it : L->items) L->key_item_begin[it.w + 1]++;
  for (int k = 0; k < nkeys; ++k) L->key_item_begin[k + 1] += L->key_item_begin[k];
  {
    // largest items first: the pair kernels' last wave then holds the
    // smallest items instead of the largest ones of the last configuration
    const int ni = (int)L->items.size();
    std::vector<double> pairs(ni, 0.0);
    for (int i = 0; i < ni; ++i) {
      const int4 it = L->items[i];
      const double na = L->tiles[it.x].y;
      for (int J = it.y; J < it.z; ++J)
        pairs[i] += (J == it.x) ? na * (na - 1) / 2 : na * L->tiles[J].y;
    }
    L->item_order.resize(ni);
    for (int i = 0; i < ni; ++i) L->item_order[i] = i;
    std::stable_sort(L->item_order.begin(), L->item_order.end(),
                     [&](int a, int b) { return pairs[a] > pairs[b]; });
  }
  {
    const int ni = (int)L->items.size(), nt = (int)L->tiles.size();
    L->adj_ioff.resize(ni);
    L->adj_joff.resize(ni);
    std::vector<std::vector<int>> per_tile(nt);
    size_t off = 0;
    for (int i = 0; i < ni; ++i) {
      const int4 it = L->items[i];
      L->adj_ioff[i] = (int)off;
      per_tile[it.x].push_back((int)off);
      off += kTile * 3;
      L->adj_joff[i] = (int)off;
      for (int T = it.y; T < it.z; ++T)
        per_tile[T].push_back((int)(off + (size_t)(T - it.y) * kTile * 3));
      off += (size_t)(it.z - it.y) * kTile * 3;
    }
    if (off > (size_t)INT32_MAX)
      return fail(ctx, PYIID_ERR_INVALID_ARG, "batch too large for the adjoint");
    L->adj_total = off;
    L->adj_tile_ptr.assign(nt + 1, 0);
    for (int t = 0; t < nt; ++t) {
      L->adj_tile_ptr[t + 1] = L->adj_tile_ptr[t] + (int)per_tile[t].size();
      L->adj_entries.insert(L->adj_entries.end(), per_tile[t].begin(),
                            per_tile[t].end());
    }
  }
  TRY(upload(ctx, &L->d_adj_ioff, L->adj_ioff));
  TRY(upload(ctx, &L->d_adj_joff, L->adj_joff));
  TRY(upload(ctx, &L->d_adj_tile_ptr, L->adj_tile_ptr));
  TRY(upload(ctx, &L->d_adj_entries, L->adj_entries));
  TRY(upload(ctx, &L->d_perm, L->perm));
  TRY(upload(ctx, &L->d_tiles, L->tiles));
  TRY(upload(ctx, &L->d_cfg_tiles, L->cfg_tiles));
  TRY(upload(ctx, &L->d_items, L->items));
  TRY(upload(ctx, &L->d_item_order, L->item_order));
  TRY(upload(ctx, &L->d_key_item_begin, L->key_item_begin));
  TRY(upload(ctx, &L->d_spair, L->spair_species));
  L->mitem_begin.push_back((int)L->mitems.size());
  TRY(upload(ctx, &L->d_mitems, L->mitems));
  TRY(upload(ctx, &L->d_mitem_begin, L->mitem_begin));
  TRY(upload(ctx, &L->d_offsets, L->offsets));
  {
    std::vector<int> sp(species, species + total);
    TRY(upload(ctx, &L->d_species, sp));
  }
  ctx->layouts.insert(ctx->layouts.begin(), std::move(L));
  while (ctx->layouts.size() > 64) {
    free_layout(ctx->layouts.back().get());
    ctx->layouts.pop_back();
  }
  *out = ctx->layouts[0].get();
  return PYIID_OK;
}

// Uploads the per-species form factor table if it changed.
int get_ftab(pyiid_ctx *ctx, const float *scatter, int n_species, int n_bins,
             float **out) {
  const size_t n = (size_t)n_species * n_bins;
  uint64_t key = fnv1a(scatter, n * sizeof(float));
  key = mix(key, n_species);
  key = mix(key, n_bins);
  void *p;
  TRY(ensure(ctx, "ftab", n * sizeof(float), &p));
  if (key != ctx->ftab_key) {
    CUDA_TRY(ctx, cudaMemcpy(p, scatter, n * sizeof(float),
                             cudaMemcpyHostToDevice));
    ctx->ftab_key = key;
  }
  *out = static_cast<float *>(p);
  return PYIID_OK;
}

// na[c][k] = N_c * (sum_sp pairs_sp f_sa f_sb) / P_c  (NaN when P_c == 0,
// as numpy's mean of an empty array).
// na_k of one configuration from its species counts:
//   n * (sum_{sa >= sb} pairs(sa, sb) f_sa f_sb) / P,  P = n (n - 1) / 2
// (NaN when P == 0).  The species-pair order is the layouts'.
void na_row(const int *count, int n_species, const float *scatter,
            int n_bins, double *row) {
  double n = 0;
  for (int sa = 0; sa < n_species; ++sa) n += count[sa];
  const double P = n * (n - 1) / 2;
  for (int k = 0; k < n_bins; ++k) {
    double s = 0.0;
    for (int sa = 0; sa < n_species; ++sa)
      for (int sb = 0; sb <= sa; ++sb) {
        const double na = count[sa], nb = count[sb];
        const double pc = (sa == sb) ? na * (na - 1) / 2 : na * nb;
        s += pc * (double)scatter[(size_t)sa * n_bins + k] *
             (double)scatter[(size_t)sb * n_bins + k];
      }
    row[k] = (P > 0) ? n * s / P : NAN;
  }
}

int get_na(pyiid_ctx *ctx, const Layout *L, const float *scatter, int n_bins,
           double **out) {
  uint64_t key = mix(L->key, ctx->ftab_key);
  key = mix(key, n_bins);
  for (size_t i = 0; i < ctx->nas.size(); ++i)
    if (ctx->nas[i]->key == key) {
      *out = ctx->nas[i]->d_na;
      return PYIID_OK;
    }
  std::vector<double> na((size_t)L->n_configs * n_bins);
  std::vector<int> count(L->n_species);
  for (int c = 0; c < L->n_configs; ++c) {
    std::fill(count.begin(), count.end(), 0);
    for (int t = L->cfg_tiles[c].x; t < L->cfg_tiles[c].y; ++t)
      count[L->tiles[t].w] += L->tiles[t].y;
    na_row(count.data(), L->n_species, scatter, n_bins,
           na.data() + (size_t)c * n_bins);
  }
  auto T = std::make_unique<NaTable>();
  T->key = key;
  TRY(upload(ctx, &T->d_na, na));
  ctx->nas.insert(ctx->nas.begin(), std::move(T));
  while (ctx->nas.size() > 64) {
    cudaFree(ctx->nas.back()->d_na);
    ctx->nas.pop_back();
  }
  *out = ctx->nas[0]->d_na;
  return PYIID_OK;
}

// The reference transform (kernels/master_kernel.py:39-203) as a matrix.
// With F' = F zeroed below kz = ceil(qmin/qstep), padded to
// len = max(n_bins, ceil(pi/rstep/qstep)), npad2 = 2 * 2^ceil(log2(
// round(qmin/qstep) + len)), the odd-extended inverse FFT gives
//   gpad[i] = (qstep/pi) sum_m F'_m sin(2 pi m i / npad2),
// and the interpolation onto r (drpad = pi/(npad2 qstep), x = r/drpad/2,
// lo = int(x), w = x - lo) gives G(r) = 2((1-w) gpad[lo] + w gpad[lo+1]), so
//   T[m][i] = (2 qstep/pi) ((1-w) sin(2 pi m lo/npad2) + w sin(2 pi m (lo+1)/npad2)).
// The sine arguments use exact integer reduction (m * lo mod npad2).
int get_tmatrix(pyiid_ctx *ctx, int n_bins, double qstep, double rstep,
                const double *rgrid, int n_r, double qmin, TMatrix **out) {
  uint64_t key = fnv1a(rgrid, sizeof(double) * (size_t)n_r);
  key = mix(key, n_bins);
  key = mix(key, qstep);
  key = mix(key, rstep);
  key = mix(key, qmin);
  for (size_t i = 0; i < ctx->tmats.size(); ++i)
    if (ctx->tmats[i]->key == key) {
      *out = ctx->tmats[i].get();
      return PYIID_OK;
    }
  if (!(qstep > 0) || !(rstep > 0))
    return fail(ctx, PYIID_ERR_INVALID_ARG, "qstep and rstep must be > 0");
  const int kz = (int)std::ceil(qmin / qstep);
  const long nfromdr = (long)std::ceil(M_PI / rstep / qstep);
  const long len = std::max<long>(n_bins, nfromdr);
  const long padrmin = (long)std::nearbyint(qmin / qstep);  // ties to even
  const long npad1 = padrmin + len;
  const long npad2 =
      (1L << (long)std::ceil(std::log((double)npad1) / std::log(2.0))) * 2;
  const double drpad = M_PI / ((double)npad2 * qstep);
  std::vector<float> T((size_t)n_bins * n_r, 0.f);
  for (int i = 0; i < n_r; ++i) {
    const double x = rgrid[i] / drpad / 2;
    const long lo = (long)x;  // truncation, as numpy astype(int)
    const double w = x - (double)lo;
    if (lo < 0 || lo + 1 >= npad2)
      return fail(ctx, PYIID_ERR_INVALID_ARG,
                  "r = %g is outside the transform range", rgrid[i]);
    for (int m = std::max(kz, 0); m < n_bins; ++m) {
      const long a = (long)(((__int128)m * lo) % npad2);
      const long b = (long)(((__int128)m * (lo + 1)) % npad2);
      const double sa = std::sin(2.0 * M_PI * (double)a / (double)npad2);
      const double sb = std::sin(2.0 * M_PI * (double)b / (double)npad2);
      T[(size_t)m * n_r + i] =
          (float)(2.0 * qstep / M_PI * ((1.0 - w) * sa + w * sb));
    }
  }
  auto M = std::make_unique<TMatrix>();
  M->key = key;
  M->n_bins = n_bins;
  M->n_r = n_r;
  M->kmin = std::max(kz, 0);
  for (size_t i = (size_t)M->kmin * n_r; i < T.size(); ++i)
    M->t_amax = std::max(M->t_amax, std::fabs(T[i]));
  TRY(upload(ctx, &M->d_T, T));
  ctx->tmats.insert(ctx->tmats.begin(), std::move(M));
  while (ctx->tmats.size() > 4) {
    free_tmatrix(ctx->tmats.back().get());
    ctx->tmats.pop_back();
  }
  *out = ctx->tmats[0].get();
  return PYIID_OK;
}

void split_double(double x, float &hi, float &lo) {
  hi = (float)x;
  lo = (float)(x - (double)hi);
}

int set_attrs(pyiid_ctx *ctx) {
  if (ctx->attrs_set) return PYIID_OK;
  for (int i = 0; i < kNumGrad; ++i)
    CUDA_TRY(ctx, cudaFuncSetAttribute(
                      kGradTable[i].k,
                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                      (int)grad_smem(kGradTable[i].v)));
  for (int i = 0; i < kNumFqGrad; ++i)
    CUDA_TRY(ctx, cudaFuncSetAttribute(
                      kFqGradTable[i].k,
                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                      (int)fqgrad_smem(kFqGradTable[i].v)));
  for (int i = 0; i < kNumFq; ++i) {
    CUDA_TRY(ctx, cudaFuncSetAttribute(
                      kFqTable[i].k,
                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                      (int)fq_smem(kFqTable[i].v)));
    if (kFqTable[i].kp)
      CUDA_TRY(ctx, cudaFuncSetAttribute(
                        kFqTable[i].kp,
                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                        (int)fq_smem(kFqTable[i].v)));
  }
  CUDA_TRY(ctx, cudaFuncSetAttribute(adjoint_sym_kernel<kAdjRS>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     160 * 1024));
  CUDA_TRY(ctx, cudaFuncSetAttribute(adjoint_kernel<kAdjRS>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     160 * 1024));
  CUDA_TRY(ctx, cudaFuncSetAttribute(move_gram_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     2 * kGramCH * 3200 * (int)sizeof(float)));
  CUDA_TRY(ctx, cudaFuncSetAttribute(
                    umma::f16x2_gemm_persistent<256, 2>,
                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                    umma::PersistShape<256, 2>::kSmem));
  CUDA_TRY(ctx, cudaFuncSetAttribute(
                    umma::f16x2_gemm_persistent<128, 3>,
                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                    umma::PersistShape<128, 3>::kSmem));
  ctx->attrs_set = true;
  return PYIID_OK;
}

// A pointer the device can write for the output `what`: device or managed
// memory as it is, pinned host memory through its device mapping (zero-copy:
// the kernel's stores cross the host link while it computes); anything
// else is rejected before any launch.
int device_view(pyiid_ctx *ctx, void *p, void **out, const char *what) {
  cudaPointerAttributes a;
  const cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, PYIID_ERR_INVALID_ARG, "%s: not a CUDA-visible pointer",
                what);
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) {
    *out = p;
    return PYIID_OK;
  }
  if (a.type == cudaMemoryTypeHost && a.devicePointer) {
    *out = a.devicePointer;
    return PYIID_OK;
  }
  return fail(ctx, PYIID_ERR_INVALID_ARG,
              "%s must be device memory or pinned, device-mapped host memory",
              what);
}

// Parts S <= min(8, n_tiles) over which the owner-computes gradient kernels
// split the tiles J of one configuration when tiles x chunk blocks CTAs give
// fewer than two waves: S minimises waves / S (each CTA's work shrinks as
// 1/S), lightly penalising the partial rows every part adds.
int choose_jsplit(pyiid_ctx *ctx, const void *kernel, int threads,
                  size_t smem, int n_tiles, int gy, int *out) {
  int per_sm = 0;
  CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &per_sm, kernel, threads, smem));
  const long long slots =
      (long long)std::max(1, per_sm) * std::max(1, ctx->n_sms);
  const long long ctas = (long long)n_tiles * gy;
  int best_s = 1;
  if (ctas < 2 * slots) {
    double best = 1e300;
    for (int S = 1; S <= std::min(kMaxJSplit, n_tiles); ++S) {
      const double waves = std::ceil((double)(ctas * S) / (double)slots);
      const double cost = waves / S * (1.0 + 0.02 * (S - 1));
      if (cost < best) {
        best = cost;
        best_s = S;
      }
    }
  }
  *out = best_s;
  return PYIID_OK;
}

// A J split of one configuration's n_tiles tiles into n parts (part p covers
// [p n_tiles / n, (p + 1) n_tiles / n)), dispatched largest part first.
JSplit make_jsplit(int n, int n_tiles, size_t out_stride, size_t fpart_stride) {
  JSplit js{n, out_stride, fpart_stride, {}};
  int idx[kMaxJSplit], size[kMaxJSplit];
  for (int p = 0; p < n && p < kMaxJSplit; ++p) {
    idx[p] = p;
    size[p] = (int)((long long)(p + 1) * n_tiles / n -
                    (long long)p * n_tiles / n);
  }
  std::stable_sort(idx, idx + std::min(n, kMaxJSplit),
                   [&](int a, int b) { return size[a] > size[b]; });
  for (int p = 0; p < kMaxJSplit; ++p)
    js.order[p] = (unsigned char)(p < n ? idx[p] : p);
  return js;
}

int check_common(pyiid_ctx *ctx, int n_configs, const int32_t *offsets,
                 int n_species, int n_bins, double qbin, int k_begin) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  if (n_configs < 1) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_configs < 1");
  if (offsets[0] != 0)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "offsets[0] must be 0");
  for (int c = 0; c < n_configs; ++c)
    if (offsets[c + 1] < offsets[c])
      return fail(ctx, PYIID_ERR_INVALID_ARG, "offsets must be non-decreasing");
  if (n_species < 1) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_species < 1");
  if (n_bins < 1) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_bins < 1");
  if (n_bins > (1 << 24))
    return fail(ctx, PYIID_ERR_INVALID_ARG, "n_bins > 2^24 is not supported");
  if (!(qbin > 0) || !std::isfinite(qbin))
    return fail(ctx, PYIID_ERR_INVALID_ARG, "qbin must be a positive number");
  if (k_begin < 0) return fail(ctx, PYIID_ERR_INVALID_ARG, "k_begin < 0");
  return PYIID_OK;
}

// Pair sums + finishing: fq[c][k] for k in [k_begin, n_bins) (zero below).
int run_fq(pyiid_ctx *ctx, const Layout *L, const float *positions,
           const float *d_ftab, const double *d_na, int n_bins, double qbin,
           int k_begin, float *fq, double *fq_raw) {
  float dq_hi, dq_lo;
  split_double(qbin, dq_hi, dq_lo);
  const int kb0 = std::min(k_begin, n_bins) & ~1;
  const int n_items = (int)L->items.size();
  double *partial = nullptr;
  if (n_items > 0 && kb0 < n_bins) {
    const FqEntry &E = kFqTable[ctx->fq_variant];
    const int Lb = E.v.L;
    const int chunks_total = (n_bins - kb0 + Lb - 1) / Lb;
    // at most 128 chunks per CTA (>= 2 pair groups) and n_chunks * L doubles
    // must fit the 32 KB record space reused by the group reduction
    const int max_chunks = std::min(128, 32768 / (8 * Lb));
    const int n_cb = (chunks_total + max_chunks - 1) / max_chunks;
    const int n_chunks = (chunks_total + n_cb - 1) / n_cb;
    const int n_groups = kBlock / n_chunks;
    void *p;
    TRY(ensure(ctx, "fq_partial", (size_t)n_items * n_bins * sizeof(double), &p));
    partial = static_cast<double *>(p);
    const size_t smem = fq_smem(E.v, n_chunks);
    if (E.kp) {
      // one launch of resident CTAs drawing work units from a counter
      void *ctr;
      TRY(ensure(ctx, "fq_counter", sizeof(int), &ctr));
      CUDA_TRY(ctx, cudaMemsetAsync(ctr, 0, sizeof(int), ctx->stream));
      int &per_sm = ctx->occupancy[{(const void *)E.kp, smem}];
      if (per_sm == 0)
        CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                          &per_sm, E.kp, kBlock, smem));
      const int n_units = n_items * n_cb;
      const int grid = std::max(
          1, std::min(n_units, std::max(per_sm, 1) * ctx->n_sms));
      E.kp<<<grid, kBlock, smem, ctx->stream>>>(
          positions, L->d_perm, L->d_tiles, L->d_items, L->d_item_order,
          dq_hi, dq_lo, kb0, n_chunks, n_groups, n_bins, n_cb, n_units,
          static_cast<int *>(ctr), partial);
    } else {
      dim3 grid(n_items, n_cb);
      E.k<<<grid, kBlock, smem, ctx->stream>>>(
          positions, L->d_perm, L->d_tiles, L->d_items, L->d_item_order,
          dq_hi, dq_lo, kb0, n_chunks, n_groups, n_bins, partial);
    }
    LAUNCH_CHECK(ctx);
  }
  dim3 g2((n_bins + 127) / 128, L->n_configs);
  const int kb_out = (n_items > 0) ? std::min(k_begin, n_bins) : n_bins;
  fq_finish_kernel<<<g2, 128, 0, ctx->stream>>>(
      partial, L->d_key_item_begin, d_ftab, L->d_spair, d_na, L->n_spairs,
      n_bins, kb_out, fq, fq_raw);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

int batch_fq(pyiid_ctx *ctx, const float *positions, const int32_t *species,
             const int32_t *offsets, int n_configs, const float *scatter,
             int n_species, int n_bins, double qbin, int k_begin, float *fq) {
  TRY(check_common(ctx, n_configs, offsets, n_species, n_bins, qbin, k_begin));
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  TRY(set_attrs(ctx));
  Layout *L;
  TRY(get_layout(ctx, species, offsets, n_configs, n_species, &L));
  float *d_ftab;
  TRY(get_ftab(ctx, scatter, n_species, n_bins, &d_ftab));
  double *d_na;
  TRY(get_na(ctx, L, scatter, n_bins, &d_na));
  return run_fq(ctx, L, positions, d_ftab, d_na, n_bins, qbin, k_begin, fq,
                nullptr);
}

}  // namespace

extern "C" {

int pyiid_version(void) { return kVersion; }

int pyiid_create(pyiid_ctx **out, int device) {
  if (!out) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null output pointer");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return fail(nullptr, PYIID_ERR_CUDA, "no CUDA device: %s",
                e == cudaSuccess ? "device count is 0" : cudaGetErrorString(e));
  if (device < 0 || device >= n)
    return fail(nullptr, PYIID_ERR_INVALID_ARG, "device %d outside [0, %d)",
                device, n);
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess)
    return fail(nullptr, PYIID_ERR_CUDA, "cudaGetDeviceProperties: %s",
                cudaGetErrorString(e));
  if (prop.major * 10 + prop.minor != 103)
    return fail(nullptr, PYIID_ERR_CUDA,
                "device %d is sm_%d%d; this library is built for sm_103a only",
                device, prop.major, prop.minor);
  e = cudaSetDevice(device);
  if (e != cudaSuccess)
    return fail(nullptr, PYIID_ERR_CUDA, "cudaSetDevice: %s",
                cudaGetErrorString(e));
  pyiid_ctx *ctx = new (std::nothrow) pyiid_ctx();
  if (!ctx) return fail(nullptr, PYIID_ERR_OOM, "out of host memory");
  ctx->device = device;
  ctx->n_sms = prop.multiProcessorCount;
  // the device status word of the kernels with bounded waits (allocated
  // here, not at first use, which may be inside a graph capture)
  if (cudaMalloc(&ctx->d_status, sizeof(int)) != cudaSuccess ||
      cudaMemset(ctx->d_status, 0, sizeof(int)) != cudaSuccess) {
    cudaFree(ctx->d_status);
    delete ctx;
    return fail(nullptr, PYIID_ERR_OOM, "cannot allocate the status word");
  }
  *out = ctx;
  return PYIID_OK;
}

}  // extern "C"
namespace {
void mlp_forget(const pyiid_ctx *ctx);
}
extern "C" {

int pyiid_destroy(pyiid_ctx *ctx) {
  if (!ctx) return PYIID_OK;
  mlp_forget(ctx);
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto &kv : ctx->bufs) cudaFree(kv.second.p);
  for (auto &L : ctx->layouts) free_layout(L.get());
  for (auto &T : ctx->tmats) free_tmatrix(T.get());
  for (auto &N : ctx->nas) cudaFree(N->d_na);
  cudaFree(ctx->d_status);
  delete ctx;
  return PYIID_OK;
}

int pyiid_set_stream(pyiid_ctx *ctx, void *stream) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  ctx->stream = static_cast<cudaStream_t>(stream);
  return PYIID_OK;
}

int pyiid_synchronize(pyiid_ctx *ctx) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->d_status) {
    int v = 0;
    CUDA_TRY(ctx, cudaMemcpy(&v, ctx->d_status, sizeof(int),
                             cudaMemcpyDeviceToHost));
    if (v) {
      CUDA_TRY(ctx, cudaMemset(ctx->d_status, 0, sizeof(int)));
      return fail(ctx, PYIID_ERR_TIMEOUT,
                  "a kernel's wait on its own pipeline gave up (code %d); "
                  "its output is not valid",
                  v);
    }
  }
  return PYIID_OK;
}

const char *pyiid_last_error(const pyiid_ctx *ctx) {
  if (ctx) return ctx->err.c_str();
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_err.c_str();
}

int64_t pyiid_launch_count(const pyiid_ctx *ctx) {
  return ctx ? ctx->launches : -1;
}

int pyiid_fq(pyiid_ctx *ctx, const float *positions, const int32_t *species,
             int n_atoms, const float *scatter, int n_species, int n_bins,
             double qbin, int k_begin, float *fq) {
  if (n_atoms < 0) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_atoms < 0");
  const int32_t offsets[2] = {0, n_atoms};
  return batch_fq(ctx, positions, species, offsets, 1, scatter, n_species,
                  n_bins, qbin, k_begin, fq);
}

int pyiid_batch_fq(pyiid_ctx *ctx, const float *positions,
                   const int32_t *species, const int32_t *offsets,
                   int n_configs, const float *scatter, int n_species,
                   int n_bins, double qbin, int k_begin, float *fq) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  if (!offsets) return fail(ctx, PYIID_ERR_INVALID_ARG, "null offsets");
  return batch_fq(ctx, positions, species, offsets, n_configs, scatter,
                  n_species, n_bins, qbin, k_begin, fq);
}

int pyiid_grad_fq(pyiid_ctx *ctx, const float *positions,
                  const int32_t *species, int n_atoms, const float *scatter,
                  int n_species, int n_bins, double qbin, int k_begin,
                  float *grad) {
  if (n_atoms < 0) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_atoms < 0");
  const int32_t offsets[2] = {0, n_atoms};
  TRY(check_common(ctx, 1, offsets, n_species, n_bins, qbin, k_begin));
  if (n_atoms == 0) return PYIID_OK;
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  TRY(set_attrs(ctx));
  Layout *L;
  TRY(get_layout(ctx, species, offsets, 1, n_species, &L));
  float *d_ftab;
  TRY(get_ftab(ctx, scatter, n_species, n_bins, &d_ftab));
  double *d_na;
  TRY(get_na(ctx, L, scatter, n_bins, &d_na));
  const int kbo = std::min(k_begin, n_bins);
  const int kb0 = kbo & ~1;
  void *p;
  TRY(ensure(ctx, "coef",
             (size_t)n_species * n_species * n_bins * sizeof(float), &p));
  float *coef = static_cast<float *>(p);
  gradfq_coef_kernel<<<64, 256, 0, ctx->stream>>>(d_na, d_ftab, n_species,
                                                  n_bins, 1, coef);
  LAUNCH_CHECK(ctx);
  int n_split = 1;
  if (kb0 < n_bins) {
    const GradEntry &E = kGradTable[ctx->grad_variant];
    const int Lb = E.v.L, cpc = E.v.CPC;
    const int chunks_total = (n_bins - kb0 + Lb - 1) / Lb;
    const int gy = (chunks_total + cpc - 1) / cpc;
    const int n_tiles = (int)L->tiles.size();
    const size_t smem = grad_smem(E.v);
    // the packed kernels split the tiles J of a small configuration (the
    // scalar ones never do)
    if (E.v.NP == 0)
      TRY(choose_jsplit(ctx, (const void *)E.k, kTile * cpc, smem, n_tiles,
                        gy, &n_split));
    const size_t gsize = (size_t)n_atoms * 3 * n_bins;
    float *gout = grad;
    if (n_split > 1) {
      TRY(ensure(ctx, "grad_gpart", (size_t)n_split * gsize * sizeof(float),
                 &p));
      gout = static_cast<float *>(p);
    }
    float dq_hi, dq_lo;
    split_double(qbin, dq_hi, dq_lo);
    dim3 grid((unsigned)n_tiles, gy, n_split);
    E.k<<<grid, kTile * cpc, smem, ctx->stream>>>(
        positions, L->d_perm, L->d_tiles, L->d_cfg_tiles, dq_hi, dq_lo, kb0,
        chunks_total, n_bins, coef, n_species, gout,
        make_jsplit(n_split, n_tiles, gsize, 0));
    LAUNCH_CHECK(ctx);
    if (n_split > 1) {
      combine_grad_parts_kernel<<<8 * std::max(1, ctx->n_sms), 256, 0,
                                  ctx->stream>>>(gout, n_split, gsize, gsize,
                                                 n_bins, kbo, grad);
      LAUNCH_CHECK(ctx);
    }
  }
  if (kbo > 0 && n_split == 1)
    CUDA_TRY(ctx, cudaMemset2DAsync(grad, (size_t)n_bins * sizeof(float), 0,
                                    (size_t)kbo * sizeof(float),
                                    (size_t)3 * n_atoms, ctx->stream));
  return PYIID_OK;
}

int pyiid_fq_grad(pyiid_ctx *ctx, const float *positions,
                  const int32_t *species, int n_atoms, const float *scatter,
                  int n_species, int n_bins, double qbin, int k_begin,
                  float *fq, float *grad) {
  if (n_atoms < 0) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_atoms < 0");
  const int32_t offsets[2] = {0, n_atoms};
  TRY(check_common(ctx, 1, offsets, n_species, n_bins, qbin, k_begin));
  if (!fq || (!grad && n_atoms > 0))
    return fail(ctx, PYIID_ERR_INVALID_ARG, "null output pointer");
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  {
    void *v;
    TRY(device_view(ctx, fq, &v, "fq"));
    fq = static_cast<float *>(v);
    if (n_atoms > 0) {
      TRY(device_view(ctx, grad, &v, "grad"));
      grad = static_cast<float *>(v);
    }
  }
  TRY(set_attrs(ctx));
  Layout *L;
  TRY(get_layout(ctx, species, offsets, 1, n_species, &L));
  float *d_ftab;
  TRY(get_ftab(ctx, scatter, n_species, n_bins, &d_ftab));
  double *d_na;
  TRY(get_na(ctx, L, scatter, n_bins, &d_na));
  const int kbo = std::min(k_begin, n_bins);
  const int kb0 = kbo & ~1;
  const int n_tiles = (int)L->tiles.size();
  double *fpart = nullptr;
  int n_split = 1;
  if (n_atoms > 0 && kb0 < n_bins) {
    void *p;
    TRY(ensure(ctx, "coef",
               (size_t)n_species * n_species * n_bins * sizeof(float), &p));
    float *coef = static_cast<float *>(p);
    gradfq_coef_kernel<<<64, 256, 0, ctx->stream>>>(d_na, d_ftab, n_species,
                                                    n_bins, 1, coef);
    LAUNCH_CHECK(ctx);
    const FqGradEntry &E = kFqGradTable[ctx->fqgrad_variant];
    const int Lb = E.v.L, cpc = E.v.CPC;
    const int chunks_total = (n_bins - kb0 + Lb - 1) / Lb;
    const int gy = (chunks_total + cpc - 1) / cpc;
    // too few CTAs for two waves: split the tiles J over n_split CTAs
    TRY(choose_jsplit(ctx, (const void *)E.k, kTile * cpc, fqgrad_smem(E.v),
                      n_tiles, gy, &n_split));
    TRY(ensure(ctx, "fqgrad_part",
               (size_t)n_split * n_tiles * n_bins * sizeof(double), &p));
    fpart = static_cast<double *>(p);
    const size_t gsize = (size_t)n_atoms * 3 * n_bins;
    float *gout = grad;
    if (n_split > 1) {
      TRY(ensure(ctx, "fqgrad_gpart", (size_t)n_split * gsize * sizeof(float),
                 &p));
      gout = static_cast<float *>(p);
    }
    float dq_hi, dq_lo;
    split_double(qbin, dq_hi, dq_lo);
    dim3 grid((unsigned)n_tiles, gy, n_split);
    E.k<<<grid, kTile * cpc, fqgrad_smem(E.v), ctx->stream>>>(
        positions, L->d_perm, L->d_tiles, L->d_cfg_tiles, dq_hi, dq_lo, kb0,
        chunks_total, n_bins, coef, n_species, gout, d_ftab, fpart, 0,
        make_jsplit(n_split, n_tiles, gsize, (size_t)n_tiles * n_bins));
    LAUNCH_CHECK(ctx);
    if (n_split > 1) {
      combine_grad_parts_kernel<<<8 * std::max(1, ctx->n_sms), 256, 0,
                                  ctx->stream>>>(gout, n_split, gsize, gsize,
                                                 n_bins, kbo, grad);
      LAUNCH_CHECK(ctx);
    }
  }
  fqgrad_finish_kernel<<<(n_bins + 3) / 4, 128, 0, ctx->stream>>>(
      fpart, 0, fpart ? n_split * n_tiles : 0, d_na, n_bins,
      fpart ? kbo : n_bins, fq, nullptr);
  LAUNCH_CHECK(ctx);
  if (kbo > 0 && n_atoms > 0 && n_split == 1)
    CUDA_TRY(ctx, cudaMemset2DAsync(grad, (size_t)n_bins * sizeof(float), 0,
                                    (size_t)kbo * sizeof(float),
                                    (size_t)3 * n_atoms, ctx->stream));
  return PYIID_OK;
}

int pyiid_fq_grad_part(pyiid_ctx *ctx, const float *positions,
                       const int32_t *species, int n_atoms,
                       const float *scatter, int n_species, int n_bins,
                       double qbin, int k_begin, int part, int n_parts,
                       double *sums, float *grad, int32_t *rows) {
  if (n_atoms < 0) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_atoms < 0");
  const int32_t offsets[2] = {0, n_atoms};
  TRY(check_common(ctx, 1, offsets, n_species, n_bins, qbin, k_begin));
  if (n_parts < 1 || part < 0 || part >= n_parts)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "part %d of %d", part, n_parts);
  if (!sums || (!grad && n_atoms > 0))
    return fail(ctx, PYIID_ERR_INVALID_ARG, "null output pointer");
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  TRY(set_attrs(ctx));
  Layout *L;
  TRY(get_layout(ctx, species, offsets, 1, n_species, &L));
  float *d_ftab;
  TRY(get_ftab(ctx, scatter, n_species, n_bins, &d_ftab));
  double *d_na;
  TRY(get_na(ctx, L, scatter, n_bins, &d_na));
  // contiguous tile range of this part, balanced by lane operations: every
  // tile sweeps all atoms for the gradient (8 per ordered pair-bin) and the
  // atoms of tiles J >= I for F(Q) (1 per pair-bin)
  const int n_tiles = (int)L->tiles.size();
  std::vector<double> cum(n_tiles + 1, 0.0), suffix(n_tiles + 1, 0.0);
  for (int t = n_tiles - 1; t >= 0; --t)
    suffix[t] = suffix[t + 1] + L->tiles[t].y;
  for (int t = 0; t < n_tiles; ++t)
    cum[t + 1] = cum[t] + (double)L->tiles[t].y *
                              (8.0 * n_atoms + suffix[t]);
  auto edge = [&](int p) {
    if (p <= 0) return 0;
    if (p >= n_parts) return n_tiles;
    const double target = cum[n_tiles] * p / n_parts;
    return (int)(std::lower_bound(cum.begin(), cum.end(), target) -
                 cum.begin());
  };
  const int t0 = std::min(edge(part), n_tiles);
  const int t1 = std::max(t0, std::min(edge(part + 1), n_tiles));
  if (rows) {
    std::fill(rows, rows + n_atoms, 0);
    for (int t = t0; t < t1; ++t)
      for (int a = 0; a < L->tiles[t].y; ++a)
        rows[L->perm[L->tiles[t].x + a]] = 1;
  }
  const int kbo = std::min(k_begin, n_bins);
  const int kb0 = kbo & ~1;
  double *fpart = nullptr;
  if (t1 > t0 && kb0 < n_bins) {
    void *p;
    TRY(ensure(ctx, "coef",
               (size_t)n_species * n_species * n_bins * sizeof(float), &p));
    float *coef = static_cast<float *>(p);
    gradfq_coef_kernel<<<64, 256, 0, ctx->stream>>>(d_na, d_ftab, n_species,
                                                    n_bins, 1, coef);
    LAUNCH_CHECK(ctx);
    TRY(ensure(ctx, "fqgrad_part", (size_t)n_tiles * n_bins * sizeof(double),
               &p));
    fpart = static_cast<double *>(p);
    const FqGradEntry &E = kFqGradTable[ctx->fqgrad_variant];
    const int Lb = E.v.L, cpc = E.v.CPC;
    const int chunks_total = (n_bins - kb0 + Lb - 1) / Lb;
    float dq_hi, dq_lo;
    split_double(qbin, dq_hi, dq_lo);
    dim3 grid((unsigned)(t1 - t0), (chunks_total + cpc - 1) / cpc);
    E.k<<<grid, kTile * cpc, fqgrad_smem(E.v), ctx->stream>>>(
        positions, L->d_perm, L->d_tiles, L->d_cfg_tiles, dq_hi, dq_lo, kb0,
        chunks_total, n_bins, coef, n_species, grad, d_ftab, fpart, t0,
        make_jsplit(1, 1, 0, 0));
    LAUNCH_CHECK(ctx);
  }
  fqgrad_finish_kernel<<<(n_bins + 3) / 4, 128, 0, ctx->stream>>>(
      fpart, t0, fpart ? t1 : t0, d_na, n_bins, kbo, nullptr, sums);
  LAUNCH_CHECK(ctx);
  if (kbo > 0 && t1 > t0) {
    zero_low_bins_kernel<<<t1 - t0, 128, 0, ctx->stream>>>(
        L->d_perm, L->d_tiles, t0, kbo, n_bins, grad);
    LAUNCH_CHECK(ctx);
  }
  return PYIID_OK;
}

int pyiid_fq_from_sums(pyiid_ctx *ctx, const int32_t *species, int n_atoms,
                       const float *scatter, int n_species, int n_bins,
                       int k_begin, const double *sums, float *fq) {
  if (n_atoms < 0) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_atoms < 0");
  const int32_t offsets[2] = {0, n_atoms};
  TRY(check_common(ctx, 1, offsets, n_species, n_bins, 1.0, k_begin));
  if (!sums || !fq)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "null pointer");
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  Layout *L;
  TRY(get_layout(ctx, species, offsets, 1, n_species, &L));
  float *d_ftab;  // keys the normalisation cache to this table
  TRY(get_ftab(ctx, scatter, n_species, n_bins, &d_ftab));
  double *d_na;
  TRY(get_na(ctx, L, scatter, n_bins, &d_na));
  const int kb_out = n_atoms > 0 ? std::min(k_begin, n_bins) : n_bins;
  fq_from_sums_kernel<<<(n_bins + 127) / 128, 128, 0, ctx->stream>>>(
      sums, d_na, n_bins, kb_out, fq);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

int pyiid_pdf(pyiid_ctx *ctx, const float *fq, int n_configs, int n_bins,
              double qstep, double rstep, const double *rgrid, int n_r,
              double qmin, double *gr) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  if (n_configs < 1 || n_bins < 1 || n_r < 0)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "bad sizes");
  if (n_r == 0) return PYIID_OK;
  if (n_bins > 12288)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "n_bins > 12288 is not supported");
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  TMatrix *T;
  TRY(get_tmatrix(ctx, n_bins, qstep, rstep, rgrid, n_r, qmin, &T));
  dim3 grid((n_r + 255) / 256, n_configs);
  pdf_kernel<<<grid, 256, n_bins * sizeof(float), ctx->stream>>>(
      fq, T->d_T, n_bins, n_r, T->kmin, gr);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

int pyiid_grad_pdf(pyiid_ctx *ctx, const float *grad_fq, int n_atoms,
                   int n_bins, double qstep, double rstep, const double *rgrid,
                   int n_r, double qmin, double *grad_pdf) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  if (n_atoms < 0 || n_bins < 1 || n_r < 0)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "bad sizes");
  if (n_atoms == 0 || n_r == 0) return PYIID_OK;
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  TMatrix *T;
  TRY(get_tmatrix(ctx, n_bins, qstep, rstep, rgrid, n_r, qmin, &T));
  TRY(set_attrs(ctx));
  const int rows = 3 * n_atoms;
  const int kw = n_bins - T->kmin;
  if (kw <= 0) {  // every bin below qmin: an all-zero product
    CUDA_TRY(ctx, cudaMemsetAsync(grad_pdf, 0,
                                  (size_t)rows * n_r * sizeof(double),
                                  ctx->stream));
    return PYIID_OK;
  }
  const int k_tiles = (kw + umma::kBK16 - 1) / umma::kBK16;
  const int m_tiles = (rows + umma::kBM - 1) / umma::kBM;
  const int a_rows_pad = m_tiles * umma::kBM;
  const int pack_grid = 8 * ctx->n_sms;
  if (!T->d_Bhi) {
    // T^T packed once per T matrix, rows padded to a multiple of 256 (the
    // widest column tile)
    T->b_rows_pad = (n_r + 255) / 256 * 256;
    T->e_t = umma::fp16_scale_exp(T->t_amax);
    const size_t nb = (size_t)k_tiles * umma::kRowBytes * T->b_rows_pad;
    CUDA_TRY(ctx, cudaMalloc(&T->d_Bhi, nb));
    CUDA_TRY(ctx, cudaMalloc(&T->d_Blo, nb));
    umma::pack_b_f16_kernel<<<pack_grid, 256, 0, ctx->stream>>>(
        T->d_T, n_bins, n_r, T->kmin, T->b_rows_pad, k_tiles, T->e_t,
        static_cast<__half *>(T->d_Bhi), static_cast<__half *>(T->d_Blo));
    LAUNCH_CHECK(ctx);
  }
  void *ahi, *alo, *rexp;
  const size_t na = (size_t)k_tiles * umma::kRowBytes * a_rows_pad;
  TRY(ensure(ctx, "gp_ahi", na, &ahi));
  TRY(ensure(ctx, "gp_alo", na, &alo));
  TRY(ensure(ctx, "gp_rexp", (size_t)a_rows_pad * sizeof(int), &rexp));
  // one warp per row (its largest magnitude, then the scaled split)
  umma::pack_a_f16_kernel<<<pack_grid, 256, 0, ctx->stream>>>(
      grad_fq, rows, n_bins, T->kmin, a_rows_pad, k_tiles,
      static_cast<__half *>(ahi), static_cast<__half *>(alo),
      static_cast<int *>(rexp));
  LAUNCH_CHECK(ctx);
  // 128 x 256 output tiles when they give every SM at least two, else
  // 128 x 128 (more CTAs for few rows); one persistent CTA per SM
  const int n256 = (n_r + 255) / 256, n128 = (n_r + 127) / 128;
  if ((long long)m_tiles * n256 >= 2LL * ctx->n_sms) {
    const int tiles = m_tiles * n256;
    umma::f16x2_gemm_persistent<256, 2>
        <<<std::min(tiles, ctx->n_sms), umma::kGemmThreads,
           umma::PersistShape<256, 2>::kSmem, ctx->stream>>>(
            ahi, alo, T->d_Bhi, T->d_Blo, k_tiles, a_rows_pad,
            T->b_rows_pad, m_tiles, n256, rows, n_r,
            static_cast<const int *>(rexp), T->e_t, grad_pdf, ctx->d_status);
  } else {
    const int tiles = m_tiles * n128;
    umma::f16x2_gemm_persistent<128, 3>
        <<<std::min(tiles, ctx->n_sms), umma::kGemmThreads,
           umma::PersistShape<128, 3>::kSmem, ctx->stream>>>(
            ahi, alo, T->d_Bhi, T->d_Blo, k_tiles, a_rows_pad,
            T->b_rows_pad, m_tiles, n128, rows, n_r,
            static_cast<const int *>(rexp), T->e_t, grad_pdf, ctx->d_status);
  }
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

int pyiid_potential(pyiid_ctx *ctx, const double *gobs, const double *gcalc,
                    int n_configs, int n_r, int potential, double *out) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  if (n_configs < 1 || n_r < 1)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "bad sizes");
  if (potential != PYIID_POTENTIAL_RW && potential != PYIID_POTENTIAL_CHI_SQ)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "unknown potential %d", potential);
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  potential_kernel<<<n_configs, 256, 0, ctx->stream>>>(gobs, gcalc, n_r,
                                                       potential, out, nullptr);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

int pyiid_potential_weighted(pyiid_ctx *ctx, const double *gobs,
                             const double *gcalc, const double *weight,
                             int n_configs, int n_r, double *out) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  if (n_configs < 1 || n_r < 1)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "bad sizes");
  if (!weight) return fail(ctx, PYIID_ERR_INVALID_ARG, "null weight");
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  potential_kernel<<<n_configs, 256, 0, ctx->stream>>>(
      gobs, gcalc, n_r, PYIID_POTENTIAL_RW, out, nullptr, weight);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

int pyiid_potential_grad(pyiid_ctx *ctx, const double *grad_pdf,
                         const double *gcalc, const double *gobs, int n_atoms,
                         int n_r, int potential, double *grad) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  if (n_atoms < 0 || n_r < 1)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "bad sizes");
  if (potential != PYIID_POTENTIAL_RW && potential != PYIID_POTENTIAL_CHI_SQ)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "unknown potential %d", potential);
  if (n_atoms == 0) return PYIID_OK;
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  void *p;
  TRY(ensure(ctx, "energy1", 2 * sizeof(double), &p));
  double *e = static_cast<double *>(p);
  TRY(ensure(ctx, "cvec", (size_t)n_r * sizeof(float), &p));
  float *cvec = static_cast<float *>(p);
  potential_kernel<<<1, 256, 0, ctx->stream>>>(gobs, gcalc, n_r, potential, e,
                                               cvec);
  LAUNCH_CHECK(ctx);
  const int rows = 3 * n_atoms;
  potential_grad_rows_kernel<<<(rows * 32 + 255) / 256, 256, 0, ctx->stream>>>(
      grad_pdf, cvec, rows, n_r, grad);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

int pyiid_batch_potential_grad(pyiid_ctx *ctx, const float *positions,
                               const int32_t *species, const int32_t *offsets,
                               int n_configs, const float *scatter,
                               int n_species, int n_bins, double qstep,
                               double rstep, const double *rgrid, int n_r,
                               double qmin, const double *gobs, int potential,
                               double *energy, float *grad, double *gcalc,
                               float *fq) {
  TRY(check_common(ctx, n_configs, offsets, n_species, n_bins, qstep, 0));
  if (n_r < 1) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_r < 1");
  if (n_bins > 12288)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "n_bins > 12288 is not supported");
  if (potential != PYIID_POTENTIAL_RW && potential != PYIID_POTENTIAL_CHI_SQ)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "unknown potential %d", potential);
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  TRY(set_attrs(ctx));
  Layout *L;
  TRY(get_layout(ctx, species, offsets, n_configs, n_species, &L));
  float *d_ftab;
  TRY(get_ftab(ctx, scatter, n_species, n_bins, &d_ftab));
  double *d_na;
  TRY(get_na(ctx, L, scatter, n_bins, &d_na));
  TMatrix *T;
  TRY(get_tmatrix(ctx, n_bins, qstep, rstep, rgrid, n_r, qmin, &T));
  const int kmin = T->kmin;
  void *p;
  float *d_fq = fq;
  if (!d_fq) {
    TRY(ensure(ctx, "b_fq", (size_t)n_configs * n_bins * sizeof(float), &p));
    d_fq = static_cast<float *>(p);
  }
  double *d_gc = gcalc;
  if (!d_gc) {
    TRY(ensure(ctx, "b_gcalc", (size_t)n_configs * n_r * sizeof(double), &p));
    d_gc = static_cast<double *>(p);
  }
  TRY(run_fq(ctx, L, positions, d_ftab, d_na, n_bins, qstep, kmin, d_fq,
             nullptr));
  dim3 gp((n_r + 255) / 256, n_configs);
  pdf_kernel<<<gp, 256, n_bins * sizeof(float), ctx->stream>>>(
      d_fq, T->d_T, n_bins, n_r, kmin, d_gc);
  LAUNCH_CHECK(ctx);
  float *cvec = nullptr;
  if (grad) {
    TRY(ensure(ctx, "b_cvec", (size_t)n_configs * n_r * sizeof(float), &p));
    cvec = static_cast<float *>(p);
  }
  potential_kernel<<<n_configs, 256, 0, ctx->stream>>>(gobs, d_gc, n_r,
                                                       potential, energy, cvec);
  LAUNCH_CHECK(ctx);
  if (!grad || L->total == 0) return PYIID_OK;
  TRY(ensure(ctx, "b_w", (size_t)n_configs * n_bins * sizeof(double), &p));
  double *w = static_cast<double *>(p);
  const int nwarps = n_configs * n_bins;
  wvec_kernel<<<(nwarps * 32 + 255) / 256, 256, 0, ctx->stream>>>(
      T->d_T, cvec, n_bins, n_r, kmin, n_configs, w);
  LAUNCH_CHECK(ctx);
  const int kb0 = kmin & ~1;
  // table length: bins [kb0, n_bins) rounded up to a multiple of 4 (two
  // packed steps); the kernel runs full re-seed blocks, then the remainder
  const int kp = std::max(4, ((n_bins - kb0 + 3) / 4) * 4);
  const size_t ntab = (size_t)n_configs * n_species * n_species * (kp / 2);
  TRY(ensure(ctx, "b_tabs", ntab * sizeof(float4), &p));
  float4 *tabs = static_cast<float4 *>(p);
  adjoint_table_kernel<<<256, 256, 0, ctx->stream>>>(
      w, d_na, d_ftab, n_species, n_bins, kmin, kb0, kp, n_configs, tabs);
  LAUNCH_CHECK(ctx);
  float dq_hi, dq_lo;
  split_double(qstep, dq_hi, dq_lo);
  const size_t smem = (size_t)n_species * (kp / 2) * sizeof(float4);
  if (smem > 160 * 1024)
    return fail(ctx, PYIID_ERR_INVALID_ARG,
                "adjoint tables (%zu bytes) exceed shared memory", smem);
  if (!L->tiles.empty() && ctx->adj_variant == 1) {
    adjoint_kernel<kAdjRS><<<(unsigned)L->tiles.size(), kBlock, smem,
                             ctx->stream>>>(positions, L->d_perm, L->d_tiles,
                                            L->d_cfg_tiles, dq_hi, dq_lo, kb0,
                                            kp, tabs, n_species, grad);
    LAUNCH_CHECK(ctx);
  } else if (!L->tiles.empty()) {
    TRY(ensure(ctx, "b_adjpart", std::max<size_t>(L->adj_total, 1) * sizeof(float),
               &p));
    float *part = static_cast<float *>(p);
    if (!L->items.empty()) {
      adjoint_sym_kernel<kAdjRS><<<(unsigned)L->items.size(), kBlock,
                                   (kp / 2) * sizeof(float4), ctx->stream>>>(
          positions, L->d_perm, L->d_tiles, L->d_items, L->d_item_order, dq_hi,
          dq_lo, kb0, kp, tabs, n_species, L->d_adj_ioff, L->d_adj_joff, part);
      LAUNCH_CHECK(ctx);
    }
    adjoint_reduce_kernel<<<(unsigned)L->tiles.size(), 96, 0, ctx->stream>>>(
        part, L->d_adj_tile_ptr, L->d_adj_entries, L->d_tiles, L->d_perm,
        (int)L->tiles.size(), grad);
    LAUNCH_CHECK(ctx);
  }
  return PYIID_OK;
}

// ------------------------------------------------- single-atom Metropolis
// Shared validation and cached tables of pyiid_mh_init / pyiid_mh_steps.
static int mh_prepare(pyiid_ctx *ctx, const int32_t *species,
                      const int32_t *offsets, int n_configs,
                      const float *scatter, int n_species, int n_bins,
                      double qstep, double rstep, const double *rgrid,
                      int n_r, double qmin, int potential, Layout **L,
                      float **ftab, double **na, TMatrix **T) {
  TRY(check_common(ctx, n_configs, offsets, n_species, n_bins, qstep, 0));
  if (n_r < 1) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_r < 1");
  if (n_bins > 12288)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "n_bins > 12288 is not supported");
  if (potential != PYIID_POTENTIAL_RW && potential != PYIID_POTENTIAL_CHI_SQ)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "unknown potential %d", potential);
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  TRY(set_attrs(ctx));
  TRY(get_layout(ctx, species, offsets, n_configs, n_species, L));
  TRY(get_ftab(ctx, scatter, n_species, n_bins, ftab));
  TRY(get_na(ctx, *L, scatter, n_bins, na));
  TRY(get_tmatrix(ctx, n_bins, qstep, rstep, rgrid, n_r, qmin, T));
  return PYIID_OK;
}

// Gram matrix of a transform (built once per T on the context stream).
static int get_gram(pyiid_ctx *ctx, TMatrix *T) {
  if (T->d_M64) return PYIID_OK;
  const size_t kk = (size_t)T->n_bins * T->n_bins;
  CUDA_TRY(ctx, cudaMalloc(&T->d_M64, kk * sizeof(double)));
  CUDA_TRY(ctx, cudaMalloc(&T->d_M32, kk * sizeof(float)));
  dim3 g((T->n_bins + 31) / 32, (T->n_bins + 31) / 32);
  gram_matrix_kernel<<<g, dim3(32, 8), 0, ctx->stream>>>(
      T->d_T, T->n_bins, T->n_r, T->d_M64, T->d_M32);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

size_t pyiid_mh_state_size(int n_configs, int n_bins) {
  if (n_configs < 0 || n_bins < 0) return 0;
  return mh_state_doubles(n_configs, n_bins);
}

int pyiid_mh_init(pyiid_ctx *ctx, const float *positions,
                  const int32_t *species, const int32_t *offsets,
                  int n_configs, const float *scatter, int n_species,
                  int n_bins, double qstep, double rstep, const double *rgrid,
                  int n_r, double qmin, const double *gobs, int potential,
                  double *state, double *energy) {
  Layout *L;
  float *d_ftab;
  double *d_na;
  TMatrix *T;
  TRY(mh_prepare(ctx, species, offsets, n_configs, scatter, n_species, n_bins,
                 qstep, rstep, rgrid, n_r, qmin, potential, &L, &d_ftab, &d_na,
                 &T));
  if (n_bins > 3200)
    return fail(ctx, PYIID_ERR_INVALID_ARG,
                "single-atom moves support at most 3200 bins");
  TRY(get_gram(ctx, T));
  const MhState st = mh_state(state, n_configs, n_bins);
  CUDA_TRY(ctx, cudaMemsetAsync(state, 0,
                                mh_state_doubles(n_configs, n_bins) *
                                    sizeof(double),
                                ctx->stream));
  TRY(run_fq(ctx, L, positions, d_ftab, d_na, n_bins, qstep, T->kmin, st.F,
             st.S));
  mh_gobs_kernel<<<n_bins + 1, 256, 0, ctx->stream>>>(T->d_T, gobs, n_bins,
                                                      n_r, st);
  LAUNCH_CHECK(ctx);
  mh_init_kernel<<<n_configs, 256, 0, ctx->stream>>>(
      T->d_M64, st, n_configs, n_bins, potential, energy);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

// Buffers and launch shapes of one single-atom step (sized before any launch,
// so that calls after the first are capturable).
struct MhStep {
  Layout *L = nullptr;
  TMatrix *T = nullptr;
  float *ftab = nullptr;
  double *na = nullptr;
  MhState st;
  MoveProposal *prop = nullptr;
  float *part = nullptr, *gpart = nullptr, *fsum = nullptr, *fdif = nullptr;
  int *done = nullptr;
  int n_configs = 0, n_bins = 0, kmin = 0, kb0 = 0, kp = 0, n_mi = 0;
  int n_cg = 0, n_rb = 0, n_cb = 0, n_chunks = 0, n_groups = 0;
  size_t smem = 0, gram_smem = 0;
  float dq_hi = 0.f, dq_lo = 0.f;
};

static int mh_step_setup(pyiid_ctx *ctx, const int32_t *species,
                         const int32_t *offsets, int n_configs,
                         const float *scatter, int n_species, int n_bins,
                         double qstep, double rstep, const double *rgrid,
                         int n_r, double qmin, int potential, double *state,
                         MhStep *S) {
  TRY(mh_prepare(ctx, species, offsets, n_configs, scatter, n_species, n_bins,
                 qstep, rstep, rgrid, n_r, qmin, potential, &S->L, &S->ftab,
                 &S->na, &S->T));
  if (!S->T->d_M64)
    return fail(ctx, PYIID_ERR_INVALID_ARG,
                "pyiid_mh_init must be called first for this grid");
  S->n_configs = n_configs;
  S->n_bins = n_bins;
  S->kmin = S->T->kmin;
  const int nkk = n_bins - S->kmin;
  if (nkk < 1 || n_bins > 3200)
    return fail(ctx, PYIID_ERR_INVALID_ARG,
                "single-atom moves need 1 to 3200 bins (and at least one "
                "above qmin)");
  S->kp = (n_bins + 3) & ~3;  // row stride of the F + F', dF rows
  S->gram_smem = 2 * (size_t)kGramCH * S->kp * sizeof(float);
  S->n_mi = (int)S->L->mitems.size();
  S->kb0 = S->kmin & ~1;
  S->st = mh_state(state, n_configs, n_bins);
  S->n_cg = (n_configs + kGramCH - 1) / kGramCH;
  S->n_rb = (nkk + kGramRB - 1) / kGramRB;
  void *p;
  TRY(ensure(ctx, "mh_prop", (size_t)n_configs * sizeof(MoveProposal), &p));
  S->prop = static_cast<MoveProposal *>(p);
  TRY(ensure(ctx, "mh_partial",
             (size_t)std::max(S->n_mi, 1) * n_bins * sizeof(float), &p));
  S->part = static_cast<float *>(p);
  TRY(ensure(ctx, "mh_done", (size_t)(n_configs + S->n_cg) * sizeof(int),
             &p));
  S->done = static_cast<int *>(p);
  TRY(ensure(ctx, "mh_gpart",
             (size_t)S->n_rb * n_configs * 2 * sizeof(float), &p));
  S->gpart = static_cast<float *>(p);
  // F + F' and dF rows; rows of chains without pair terms stay zero
  TRY(ensure(ctx, "mh_fsd", 2 * (size_t)n_configs * S->kp * sizeof(float),
             &p));
  S->fsum = static_cast<float *>(p);
  S->fdif = S->fsum + (size_t)n_configs * S->kp;
  // chunks of kMoveL bins; at most 16 chunks per CTA (>= 16 atom groups)
  const int chunks_total =
      std::max(1, (n_bins - S->kb0 + kMoveL - 1) / kMoveL);
  S->n_cb = (chunks_total + 15) / 16;
  S->n_chunks = (chunks_total + S->n_cb - 1) / S->n_cb;
  S->n_groups = kBlock / S->n_chunks;
  S->smem = 4 * kMoveTiles * kTile * sizeof(float4) +
            (size_t)kMoveL * (kBlock + 1) * sizeof(float);
  split_double(qstep, S->dq_hi, S->dq_lo);
  return PYIID_OK;
}

// Counters and spare rows start at zero for each call.
static int mh_step_reset(pyiid_ctx *ctx, const MhStep &S) {
  CUDA_TRY(ctx, cudaMemsetAsync(S.done, 0,
                                (size_t)(S.n_configs + S.n_cg) * sizeof(int),
                                ctx->stream));
  CUDA_TRY(ctx, cudaMemsetAsync(S.fsum, 0,
                                2 * (size_t)S.n_configs * S.kp * sizeof(float),
                                ctx->stream));
  return PYIID_OK;
}

static int mh_step_launch(pyiid_ctx *ctx, const MhStep &S, float *positions,
                          uint64_t *counter, uint64_t seed, float sigma,
                          HostMoves hm, int potential, double beta,
                          double *energy, int64_t *accepted, double *trace,
                          double *eval_out) {
  if (S.n_mi > 0) {
    dim3 g1(S.n_mi, S.n_cb);
    move_delta_kernel<<<g1, kBlock, S.smem, ctx->stream>>>(
        positions, S.L->d_perm, S.L->d_tiles, S.L->d_mitems,
        S.L->d_mitem_begin, S.L->d_offsets, S.L->d_species,
        reinterpret_cast<const unsigned long long *>(counter), (uint32_t)seed,
        (uint32_t)(seed >> 32), sigma, S.dq_hi, S.dq_lo, S.kb0, S.kmin,
        S.n_chunks, S.n_groups, S.n_bins, S.ftab, S.na, S.st, S.n_configs,
        S.kp, hm, S.prop, S.part, S.done, S.fsum, S.fdif);
    LAUNCH_CHECK(ctx);
  }
  dim3 gg(S.n_rb, S.n_cg);
  move_gram_kernel<<<gg, 256, S.gram_smem, ctx->stream>>>(
      S.T->d_M32, S.fsum, S.fdif, S.kp, S.L->d_offsets, S.prop, S.st,
      S.n_configs, S.n_bins, S.kmin, potential, beta, S.gpart,
      S.done + S.n_configs, positions, energy,
      reinterpret_cast<unsigned long long *>(counter),
      reinterpret_cast<long long *>(accepted), trace, eval_out);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

int pyiid_mh_steps(pyiid_ctx *ctx, float *positions, const int32_t *species,
                   const int32_t *offsets, int n_configs, const float *scatter,
                   int n_species, int n_bins, double qstep, double rstep,
                   const double *rgrid, int n_r, double qmin, int potential,
                   double conv, double kT, float sigma, uint64_t seed,
                   int n_steps, double *state, double *energy,
                   uint64_t *counter, int64_t *accepted, double *trace) {
  if (!(kT > 0) || !std::isfinite(kT))
    return fail(ctx, PYIID_ERR_INVALID_ARG, "kT must be a positive number");
  if (!std::isfinite(conv))
    return fail(ctx, PYIID_ERR_INVALID_ARG, "conv must be finite");
  if (!(sigma >= 0) || !std::isfinite(sigma))
    return fail(ctx, PYIID_ERR_INVALID_ARG, "sigma must be >= 0");
  if (n_steps < 0) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_steps < 0");
  MhStep S;
  TRY(mh_step_setup(ctx, species, offsets, n_configs, scatter, n_species,
                    n_bins, qstep, rstep, rgrid, n_r, qmin, potential, state,
                    &S));
  if (n_steps == 0) return PYIID_OK;
  TRY(mh_step_reset(ctx, S));
  const double beta = conv / kT;
  for (int step = 0; step < n_steps; ++step)
    TRY(mh_step_launch(ctx, S, positions, counter, seed, sigma, HostMoves{},
                       potential, beta, energy, accepted,
                       trace ? trace + (size_t)step * n_configs * 8 : nullptr,
                       nullptr));
  return PYIID_OK;
}

int pyiid_mc_propose(pyiid_ctx *ctx, const float *positions,
                     const int32_t *species, const int32_t *offsets,
                     int n_configs, const float *scatter, int n_species,
                     int n_bins, double qstep, double rstep,
                     const double *rgrid, int n_r, double qmin, int potential,
                     const int32_t *mode, const int32_t *atom,
                     const float *xyz, const int32_t *new_species,
                     double *state, double *eval) {
  MhStep S;
  TRY(mh_step_setup(ctx, species, offsets, n_configs, scatter, n_species,
                    n_bins, qstep, rstep, rgrid, n_r, qmin, potential, state,
                    &S));
  std::vector<int4> hp(n_configs);
  std::vector<float4> hx(n_configs);
  std::vector<double> na((size_t)n_configs * n_bins);
  std::vector<int> count(n_species);
  for (int c = 0; c < n_configs; ++c) {
    const int o0 = offsets[c], n = offsets[c + 1] - offsets[c];
    const int m = mode[c];
    if (m != kMoveDisplace && m != kMoveInsert && m != kMoveRemove)
      return fail(ctx, PYIID_ERR_INVALID_ARG, "mode[%d] = %d is unknown", c, m);
    if (m == kMoveInsert && n < 1)
      return fail(ctx, PYIID_ERR_INVALID_ARG,
                  "insertion into configuration %d needs at least one atom", c);
    if (m == kMoveInsert &&
        (new_species[c] < 0 || new_species[c] >= n_species))
      return fail(ctx, PYIID_ERR_INVALID_ARG,
                  "new_species[%d] = %d outside [0, %d)", c, new_species[c],
                  n_species);
    if (m != kMoveInsert && (atom[c] < 0 || atom[c] >= n))
      return fail(ctx, PYIID_ERR_INVALID_ARG,
                  "atom[%d] = %d outside configuration %d (%d atoms)", c,
                  atom[c], c, n);
    if (m == kMoveRemove && n < 2)
      return fail(ctx, PYIID_ERR_INVALID_ARG,
                  "removal from configuration %d needs at least two atoms", c);
    hp[c] = make_int4(m, m == kMoveInsert ? 0 : atom[c],
                      m == kMoveInsert ? new_species[c] : 0, 0);
    hx[c] = make_float4(m == kMoveRemove ? 0.f : xyz[3 * c],
                        m == kMoveRemove ? 0.f : xyz[3 * c + 1],
                        m == kMoveRemove ? 0.f : xyz[3 * c + 2], 0.f);
    std::fill(count.begin(), count.end(), 0);
    for (int i = o0; i < o0 + n; ++i) count[species[i]]++;
    if (m == kMoveInsert) count[new_species[c]]++;
    if (m == kMoveRemove) count[species[o0 + atom[c]]]--;
    na_row(count.data(), n_species, scatter, n_bins,
           na.data() + (size_t)c * n_bins);
  }
  void *p;
  TRY(ensure(ctx, "mc_prop", (size_t)n_configs * sizeof(int4), &p));
  int4 *d_hp = static_cast<int4 *>(p);
  TRY(ensure(ctx, "mc_xyz", (size_t)n_configs * sizeof(float4), &p));
  float4 *d_hx = static_cast<float4 *>(p);
  TRY(ensure(ctx, "mc_na", na.size() * sizeof(double), &p));
  double *d_na = static_cast<double *>(p);
  CUDA_TRY(ctx, cudaMemcpyAsync(d_hp, hp.data(), hp.size() * sizeof(int4),
                                cudaMemcpyHostToDevice, ctx->stream));
  CUDA_TRY(ctx, cudaMemcpyAsync(d_hx, hx.data(), hx.size() * sizeof(float4),
                                cudaMemcpyHostToDevice, ctx->stream));
  CUDA_TRY(ctx, cudaMemcpyAsync(d_na, na.data(), na.size() * sizeof(double),
                                cudaMemcpyHostToDevice, ctx->stream));
  TRY(mh_step_reset(ctx, S));
  HostMoves hm{d_hp, d_hx, d_na};
  TRY(mh_step_launch(ctx, S, const_cast<float *>(positions), nullptr, 0, 0.f,
                     hm, potential, 1.0, nullptr, nullptr, nullptr, eval));
  // the host arrays above are read by the copies: wait before returning
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return PYIID_OK;
}

int pyiid_mc_accept(pyiid_ctx *ctx, const int32_t *accept, int n_configs,
                    int n_bins, const double *eval, double *state,
                    double *energy) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  if (n_configs < 1) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_configs < 1");
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  void *p;
  TRY(ensure(ctx, "mc_accept", (size_t)n_configs * sizeof(int), &p));
  int *d_acc = static_cast<int *>(p);
  CUDA_TRY(ctx, cudaMemcpyAsync(d_acc, accept, (size_t)n_configs * sizeof(int),
                                cudaMemcpyHostToDevice, ctx->stream));
  mh_commit_kernel<<<(n_configs + 127) / 128, 128, 0, ctx->stream>>>(
      d_acc, eval, mh_state(state, n_configs, n_bins), energy, n_configs);
  LAUNCH_CHECK(ctx);
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return PYIID_OK;
}

// ------------------------------------------------------------------ springs
static int spring_check(pyiid_ctx *ctx, int n_atoms, double k, double rt,
                        int sp_type, const double *com) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  if (n_atoms < 0) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_atoms < 0");
  if (!std::isfinite(k) || !std::isfinite(rt))
    return fail(ctx, PYIID_ERR_INVALID_ARG, "k and rt must be finite");
  if (sp_type < PYIID_SPRING_REP || sp_type > PYIID_SPRING_COM)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "unknown spring type %d", sp_type);
  if (sp_type == PYIID_SPRING_COM && !com)
    return fail(ctx, PYIID_ERR_INVALID_ARG,
                "the centre-of-mass spring needs com");
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  return PYIID_OK;
}

int pyiid_spring(pyiid_ctx *ctx, const float *positions, int n_atoms,
                 double k, double rt, int sp_type, const double *com,
                 double *energy, float *forces, double *atomwise) {
  TRY(spring_check(ctx, n_atoms, k, rt, sp_type, com));
  const int nb = std::max(1, (n_atoms + kSpringBlock - 1) / kSpringBlock);
  void *p;
  TRY(ensure(ctx, "spring_part", 2 * (size_t)nb * sizeof(double), &p));
  double *part = static_cast<double *>(p);
  if (n_atoms == 0) {
    CUDA_TRY(ctx, cudaMemsetAsync(energy, 0, sizeof(double), ctx->stream));
    if (atomwise && sp_type == PYIID_SPRING_COM)
      CUDA_TRY(ctx, cudaMemsetAsync(atomwise, 0, sizeof(double), ctx->stream));
    return PYIID_OK;
  }
  if (sp_type == PYIID_SPRING_COM) {
    com_spring_kernel<<<nb, kSpringBlock, 0, ctx->stream>>>(
        positions, n_atoms, (float)k, (float)rt, com[0], com[1], com[2], part,
        part + nb, forces);
    LAUNCH_CHECK(ctx);
    if (atomwise) {
      sum_partials_kernel<<<1, 256, 0, ctx->stream>>>(part + nb, nb, atomwise);
      LAUNCH_CHECK(ctx);
    }
  } else {
    spring_pair_kernel<<<nb, kSpringBlock, 0, ctx->stream>>>(
        positions, n_atoms, (float)k, (float)rt, sp_type, part, forces,
        atomwise);
    LAUNCH_CHECK(ctx);
  }
  sum_partials_kernel<<<1, 256, 0, ctx->stream>>>(part, nb, energy);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

int pyiid_spring_voxels(pyiid_ctx *ctx, const float *positions, int n_atoms,
                        double k, double rt, int sp_type, const double *com,
                        int nx, int ny, int nz, double resolution,
                        double *voxels) {
  TRY(spring_check(ctx, n_atoms, k, rt, sp_type, com));
  if (nx < 0 || ny < 0 || nz < 0)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "negative voxel grid");
  if (!(resolution > 0) || !std::isfinite(resolution))
    return fail(ctx, PYIID_ERR_INVALID_ARG, "resolution must be > 0");
  const long long nv = (long long)nx * ny * nz;
  if (nv == 0) return PYIID_OK;
  const long long nb = (nv + kSpringBlock - 1) / kSpringBlock;
  if (nb > INT32_MAX)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "voxel grid too large");
  const double c0 = com ? com[0] : 0.0, c1 = com ? com[1] : 0.0,
               c2 = com ? com[2] : 0.0;
  spring_voxel_kernel<<<(unsigned)nb, kSpringBlock, 0, ctx->stream>>>(
      positions, n_atoms, (float)k, (float)rt, sp_type, c0, c1, c2, nx, ny, nz,
      (float)resolution, voxels);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

int pyiid_variant_count(int kernel) {
  switch (kernel) {
    case PYIID_KERNEL_FQ:
      return kNumFq;
    case PYIID_KERNEL_GRAD_FQ:
      return kNumGrad;
    case PYIID_KERNEL_ADJOINT:
      return 2;
    case PYIID_KERNEL_FQ_GRAD:
      return kNumFqGrad;
    case PYIID_KERNEL_MLP:
      return 3;
    default:
      return -1;
  }
}

int pyiid_variant_info(int kernel, int variant, int *params, int n_params) {
  if (!params || n_params < 3)
    return fail(nullptr, PYIID_ERR_INVALID_ARG, "params must hold 3 ints");
  if (kernel == PYIID_KERNEL_FQ && variant >= 0 && variant < kNumFq) {
    params[0] = kFqTable[variant].v.L;
    params[1] = kFqTable[variant].v.NP;
    params[2] = kBlock;
    return PYIID_OK;
  }
  if (kernel == PYIID_KERNEL_GRAD_FQ && variant >= 0 && variant < kNumGrad) {
    params[0] = kGradTable[variant].v.L;
    params[1] = kGradTable[variant].v.NP;
    params[2] = kTile * kGradTable[variant].v.CPC;
    return PYIID_OK;
  }
  if (kernel == PYIID_KERNEL_FQ_GRAD && variant >= 0 && variant < kNumFqGrad) {
    params[0] = kFqGradTable[variant].v.L;
    params[1] = kFqGradTable[variant].v.NP;
    params[2] = kTile * kFqGradTable[variant].v.CPC;
    return PYIID_OK;
  }
  if (kernel == PYIID_KERNEL_MLP && variant >= 0 && variant <= 2) {
    // atoms in flight per CTA (per warp for mma.sync), tensor memory used,
    // threads per CTA
    const int info[3][3] = {{16, 0, 256}, {128, 1, 128}, {256, 1, 512}};
    for (int i = 0; i < 3; ++i) params[i] = info[variant][i];
    return PYIID_OK;
  }
  if (kernel == PYIID_KERNEL_ADJOINT && (variant == 0 || variant == 1)) {
    params[0] = kAdjRS;               // bins between re-seeds
    params[1] = variant == 0 ? 1 : 2; // evaluations per unordered pair
    params[2] = kBlock;
    return PYIID_OK;
  }
  return fail(nullptr, PYIID_ERR_INVALID_ARG, "unknown kernel %d variant %d",
              kernel, variant);
}

int pyiid_set_variant(pyiid_ctx *ctx, int kernel, int variant) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  const int n = pyiid_variant_count(kernel);
  if (n < 0 || variant < 0 || variant >= n)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "unknown kernel %d variant %d",
                kernel, variant);
  if (kernel == PYIID_KERNEL_FQ)
    ctx->fq_variant = variant;
  else if (kernel == PYIID_KERNEL_GRAD_FQ)
    ctx->grad_variant = variant;
  else if (kernel == PYIID_KERNEL_FQ_GRAD)
    ctx->fqgrad_variant = variant;
  else if (kernel == PYIID_KERNEL_MLP)
    ctx->mlp_variant = variant;
  else
    ctx->adj_variant = variant;
  return PYIID_OK;
}

int pyiid_get_variant(const pyiid_ctx *ctx, int kernel) {
  if (!ctx) return -1;
  if (kernel == PYIID_KERNEL_FQ) return ctx->fq_variant;
  if (kernel == PYIID_KERNEL_GRAD_FQ) return ctx->grad_variant;
  if (kernel == PYIID_KERNEL_ADJOINT) return ctx->adj_variant;
  if (kernel == PYIID_KERNEL_FQ_GRAD) return ctx->fqgrad_variant;
  if (kernel == PYIID_KERNEL_MLP) return ctx->mlp_variant;
  return -1;
}

}  // extern "C"

// ===================================================================== F(Q)
// without device allocation.
//
// Some callers cannot allocate device memory: code running inside a CUDA
// graph capture or a pre-reserved memory pool, inference servers whose
// allocator owns all device memory, or embedded hosts without a device
// allocator at all.  pyiid_fq_noalloc computes exactly what pyiid_fq computes
// but keeps every device-side intermediate (atom order, tiles, work items,
// form factors, normalisation, per-item partial sums) in one file-scope
// device array of fixed size instead of context workspace buffers.
namespace {

constexpr size_t kNoAllocBytes = 32u << 20;  // 32 MiB, held per loaded device
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {};  // device address of the array, per device

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

extern "C" int pyiid_fq_noalloc(pyiid_ctx *ctx, const float *positions,
                                const int32_t *species, int n_atoms,
                                const float *scatter, int n_species,
                                int n_bins, double qbin, int k_begin,
                                float *fq) {
  if (n_atoms < 0) return fail(ctx, PYIID_ERR_INVALID_ARG, "n_atoms < 0");
  const int32_t offsets[2] = {0, n_atoms};
  TRY(check_common(ctx, 1, offsets, n_species, n_bins, qbin, k_begin));
  if (ctx->device < 0 || ctx->device >= 64)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "device id %d >= 64", ctx->device);
  for (int i = 0; i < n_atoms; ++i)
    if (species[i] < 0 || species[i] >= n_species)
      return fail(ctx, PYIID_ERR_INVALID_ARG,
                  "species[%d] = %d outside [0, %d)", i, species[i], n_species);
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  TRY(set_attrs(ctx));
  // one-time set-up per device: the device address of the scratch array
  void *base;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[ctx->device]) {
      void *p = nullptr;
      CUDA_TRY(ctx, cudaGetSymbolAddress(&p, g_noalloc_scratch));
      g_noalloc_ptr[ctx->device] = p;
    }
    base = g_noalloc_ptr[ctx->device];
  }
  // host-side layout of the single configuration (same rules as get_layout)
  const int n_spairs = n_species * (n_species + 1) / 2;
  std::vector<int> count(n_species, 0), start(n_species, 0), perm(n_atoms);
  for (int i = 0; i < n_atoms; ++i) count[species[i]]++;
  for (int s = 1; s < n_species; ++s) start[s] = start[s - 1] + count[s - 1];
  {
    std::vector<int> fillp = start;
    for (int i = 0; i < n_atoms; ++i) perm[fillp[species[i]]++] = i;
  }
  std::vector<int4> tiles;
  for (int s = 0; s < n_species; ++s)
    for (int a = 0; a < count[s]; a += kTile)
      tiles.push_back(make_int4(start[s] + a, std::min(kTile, count[s] - a), 0, s));
  std::vector<int4> items;
  // runs of J tiles as get_layout cuts them: shorter than kJMax when that
  // would leave fewer than about four work items per SM
  const double n_t = (double)tiles.size();
  const int jmax = std::max(
      1, std::min(kJMax, (int)std::floor(n_t * (n_t + 1) / 2 /
                                         (4.0 * std::max(1, ctx->n_sms)))));
  for (int I = 0; I < (int)tiles.size(); ++I) {
    int J = 0;
    while (J <= I) {
      const int sJ = tiles[J].w;
      int Je = J;
      while (Je <= I && tiles[Je].w == sJ && Je - J < jmax) ++Je;
      const int sI = tiles[I].w;
      items.push_back(make_int4(I, J, Je, sI * (sI + 1) / 2 + sJ));
      J = Je;
    }
  }
  std::stable_sort(items.begin(), items.end(),
                   [](const int4 &a, const int4 &b) { return a.w < b.w; });
  std::vector<int> key_begin(n_spairs + 1, 0);
  for (const int4 &it : items) key_begin[it.w + 1]++;
  for (int k = 0; k < n_spairs; ++k) key_begin[k + 1] += key_begin[k];
  std::vector<int2> spair;
  for (int sa = 0; sa < n_species; ++sa)
    for (int sb = 0; sb <= sa; ++sb) spair.push_back(make_int2(sa, sb));
  std::vector<double> na(n_bins);
  {
    const double n = n_atoms, P = n * (n - 1) / 2;
    for (int k = 0; k < n_bins; ++k) {
      double s = 0.0;
      for (int sp = 0; sp < n_spairs; ++sp) {
        const int sa = spair[sp].x, sb = spair[sp].y;
        const double pc = (sa == sb) ? (double)count[sa] * (count[sa] - 1) / 2
                                     : (double)count[sa] * count[sb];
        s += pc * (double)scatter[(size_t)sa * n_bins + k] *
             (double)scatter[(size_t)sb * n_bins + k];
      }
      na[k] = (P > 0) ? n * s / P : NAN;
    }
  }
  // carve the scratch array
  const int n_items = (int)items.size();
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    size_t o = off;
    off = align256(off + std::max<size_t>(bytes, 1));
    return o;
  };
  const size_t o_perm = carve(sizeof(int) * perm.size());
  const size_t o_tiles = carve(sizeof(int4) * tiles.size());
  const size_t o_items = carve(sizeof(int4) * items.size());
  const size_t o_keys = carve(sizeof(int) * key_begin.size());
  const size_t o_spair = carve(sizeof(int2) * spair.size());
  const size_t o_ftab = carve(sizeof(float) * (size_t)n_species * n_bins);
  const size_t o_na = carve(sizeof(double) * (size_t)n_bins);
  const size_t o_part = carve(sizeof(double) * (size_t)n_items * n_bins);
  if (off > kNoAllocBytes)
    return fail(ctx, PYIID_ERR_INVALID_ARG,
                "pyiid_fq_noalloc needs %zu bytes of scratch for %d atoms x %d "
                "bins; the fixed scratch array holds %zu bytes (use pyiid_fq)",
                off, n_atoms, n_bins, kNoAllocBytes);
  unsigned char *sb = static_cast<unsigned char *>(base);
  int *d_perm = reinterpret_cast<int *>(sb + o_perm);
  int4 *d_tiles = reinterpret_cast<int4 *>(sb + o_tiles);
  int4 *d_items = reinterpret_cast<int4 *>(sb + o_items);
  int *d_keys = reinterpret_cast<int *>(sb + o_keys);
  int2 *d_spair = reinterpret_cast<int2 *>(sb + o_spair);
  float *d_ftab = reinterpret_cast<float *>(sb + o_ftab);
  double *d_na = reinterpret_cast<double *>(sb + o_na);
  double *d_part = reinterpret_cast<double *>(sb + o_part);
  cudaStream_t st = ctx->stream;
  // synchronous-to-host copies: the host vectors die at return
  if (!perm.empty())
    CUDA_TRY(ctx, cudaMemcpyAsync(d_perm, perm.data(), sizeof(int) * perm.size(),
                                  cudaMemcpyHostToDevice, st));
  if (!tiles.empty())
    CUDA_TRY(ctx, cudaMemcpyAsync(d_tiles, tiles.data(),
                                  sizeof(int4) * tiles.size(),
                                  cudaMemcpyHostToDevice, st));
  if (!items.empty())
    CUDA_TRY(ctx, cudaMemcpyAsync(d_items, items.data(),
                                  sizeof(int4) * items.size(),
                                  cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(d_keys, key_begin.data(),
                                sizeof(int) * key_begin.size(),
                                cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(d_spair, spair.data(),
                                sizeof(int2) * spair.size(),
                                cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(d_ftab, scatter,
                                sizeof(float) * (size_t)n_species * n_bins,
                                cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(d_na, na.data(), sizeof(double) * na.size(),
                                cudaMemcpyHostToDevice, st));
  // pair sums into the partial rows, then the FP64 finish (as run_fq does)
  float dq_hi, dq_lo;
  split_double(qbin, dq_hi, dq_lo);
  const int kb0 = std::min(k_begin, n_bins) & ~1;
  if (n_items > 0 && kb0 < n_bins) {
    const FqEntry &E = kFqTable[ctx->fq_variant];
    const int Lb = E.v.L;
    const int chunks_total = (n_bins - kb0 + Lb - 1) / Lb;
    const int max_chunks = std::min(128, 32768 / (8 * Lb));
    const int n_cb = (chunks_total + max_chunks - 1) / max_chunks;
    const int n_chunks = (chunks_total + n_cb - 1) / n_cb;
    const int n_groups = kBlock / n_chunks;
    dim3 grid(n_items, n_cb);
    E.k<<<grid, kBlock, fq_smem(E.v, n_chunks), st>>>(
        positions, d_perm, d_tiles, d_items, nullptr, dq_hi, dq_lo, kb0,
        n_chunks, n_groups, n_bins, d_part);
    LAUNCH_CHECK(ctx);
  }
  dim3 g2((n_bins + 127) / 128, 1);
  const int kb_out = (n_items > 0) ? std::min(k_begin, n_bins) : n_bins;
  fq_finish_kernel<<<g2, 128, 0, st>>>(d_part, d_keys, d_ftab, d_spair, d_na,
                                       n_spairs, n_bins, kb_out, fq, nullptr);
  LAUNCH_CHECK(ctx);
  // the host vectors are released on return: wait for the copies only
  CUDA_TRY(ctx, cudaStreamSynchronize(st));
  return PYIID_OK;
}

// =============================================================== surrogate
// Radial-basis descriptors and the per-atom MLP of the delayed-acceptance
// surrogate.  The forward pass keeps its activations in the context
// workspace; pyiid_mlp_backward differentiates the most recent forward.
#include "surrogate_kernels.cuh"
#include "mlp_tc.cuh"

namespace {

struct MlpState {
  int n_atoms = 0, n_in = 0, n_hidden = 0, n_configs = 0;
  const __nv_bfloat16 *feat = nullptr, *w1 = nullptr, *w2 = nullptr;
  const float *w3 = nullptr;
  int *atom_cfg = nullptr;
  uint64_t cfg_key = 0;
};
std::mutex g_mlp_mu;
std::unordered_map<const pyiid_ctx *, MlpState> g_mlp;

void mlp_forget(const pyiid_ctx *ctx) {
  std::lock_guard<std::mutex> lk(g_mlp_mu);
  g_mlp.erase(ctx);
}

// atom -> configuration map and offsets on the device (cached by content)
int config_map(pyiid_ctx *ctx, const int32_t *offsets, int n_configs,
               int **d_cfg, int **d_off) {
  const int total = offsets[n_configs];
  uint64_t key = fnv1a(offsets, sizeof(int32_t) * (n_configs + 1));
  void *p;
  TRY(ensure(ctx, "sg_cfg", sizeof(int) * std::max(total, 1), &p));
  *d_cfg = static_cast<int *>(p);
  TRY(ensure(ctx, "sg_off", sizeof(int) * (n_configs + 1), &p));
  *d_off = static_cast<int *>(p);
  std::lock_guard<std::mutex> lk(g_mlp_mu);
  MlpState &S = g_mlp[ctx];
  if (S.cfg_key != key || S.atom_cfg != *d_cfg) {
    std::vector<int> cfg(std::max(total, 1), 0);
    for (int c = 0; c < n_configs; ++c)
      for (int a = offsets[c]; a < offsets[c + 1]; ++a) cfg[a] = c;
    CUDA_TRY(ctx, cudaMemcpy(*d_cfg, cfg.data(), sizeof(int) * cfg.size(),
                             cudaMemcpyHostToDevice));
    CUDA_TRY(ctx, cudaMemcpy(*d_off, offsets, sizeof(int) * (n_configs + 1),
                             cudaMemcpyHostToDevice));
    S.cfg_key = key;
    S.atom_cfg = *d_cfg;
  }
  return PYIID_OK;
}

template <bool TA, bool TB>
int gemm(pyiid_ctx *ctx, const __nv_bfloat16 *A, int lda,
         const __nv_bfloat16 *B, int ldb, float *C, int ldc, int M, int N,
         int K, int accumulate) {
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  gemm_bf16_kernel<TA, TB><<<grid, 128, 0, ctx->stream>>>(A, lda, B, ldb, C,
                                                          ldc, M, N, K,
                                                          accumulate);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

int check_offsets(pyiid_ctx *ctx, const int32_t *offsets, int n_configs) {
  if (!offsets || n_configs < 1 || offsets[0] != 0)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "bad offsets");
  for (int c = 0; c < n_configs; ++c)
    if (offsets[c + 1] < offsets[c])
      return fail(ctx, PYIID_ERR_INVALID_ARG, "offsets must be non-decreasing");
  return PYIID_OK;
}

}  // namespace

extern "C" int pyiid_rbf_features(pyiid_ctx *ctx, const float *positions,
                                  const int32_t *offsets, int n_configs,
                                  int n_centres, float r_cut, float sigma,
                                  void *feat_bf16, float *feat_f32) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  TRY(check_offsets(ctx, offsets, n_configs));
  if (n_centres < 2 || n_centres > 64)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "n_centres must be in [2, 64]");
  if (!(r_cut > 0) || !(sigma > 0))
    return fail(ctx, PYIID_ERR_INVALID_ARG, "r_cut and sigma must be > 0");
  const int total = offsets[n_configs];
  if (total == 0) return PYIID_OK;
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  int *d_cfg, *d_off;
  TRY(config_map(ctx, offsets, n_configs, &d_cfg, &d_off));
  const int warps = 8;
  rbf_features_kernel<<<(total + warps - 1) / warps, 32 * warps, 0,
                        ctx->stream>>>(
      positions, d_cfg, d_off, total, n_centres, r_cut, sigma,
      static_cast<__nv_bfloat16 *>(feat_bf16), feat_f32);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

extern "C" int pyiid_mlp_forward(pyiid_ctx *ctx, const void *feat_bf16,
                                 int n_atoms, int n_in, const int32_t *offsets,
                                 int n_configs, const void *w1_bf16,
                                 const float *b1, const void *w2_bf16,
                                 const float *b2, const float *w3,
                                 const float *b3, int n_hidden,
                                 double *energy) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  TRY(check_offsets(ctx, offsets, n_configs));
  if (offsets[n_configs] != n_atoms)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "offsets[n_configs] != n_atoms");
  if (n_in < 1 || n_hidden < 1)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "bad layer sizes");
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  int *d_cfg, *d_off;
  TRY(config_map(ctx, offsets, n_configs, &d_cfg, &d_off));
  const size_t nh = (size_t)std::max(n_atoms, 1) * n_hidden;
  void *p;
  TRY(ensure(ctx, "sg_h1", nh * sizeof(float), &p));
  float *h1 = static_cast<float *>(p);
  TRY(ensure(ctx, "sg_pre1", nh * sizeof(float), &p));
  float *pre1 = static_cast<float *>(p);
  TRY(ensure(ctx, "sg_h1b", nh * sizeof(__nv_bfloat16), &p));
  __nv_bfloat16 *h1b = static_cast<__nv_bfloat16 *>(p);
  TRY(ensure(ctx, "sg_h2", nh * sizeof(float), &p));
  float *h2 = static_cast<float *>(p);
  TRY(ensure(ctx, "sg_pre2", nh * sizeof(float), &p));
  float *pre2 = static_cast<float *>(p);
  TRY(ensure(ctx, "sg_h2b", nh * sizeof(__nv_bfloat16), &p));
  __nv_bfloat16 *h2b = static_cast<__nv_bfloat16 *>(p);
  TRY(ensure(ctx, "sg_y", sizeof(float) * std::max(n_atoms, 1), &p));
  float *y = static_cast<float *>(p);
  const __nv_bfloat16 *X = static_cast<const __nv_bfloat16 *>(feat_bf16);
  const __nv_bfloat16 *W1 = static_cast<const __nv_bfloat16 *>(w1_bf16);
  const __nv_bfloat16 *W2 = static_cast<const __nv_bfloat16 *>(w2_bf16);
  if (n_atoms > 0) {
    TRY((gemm<false, false>(ctx, X, n_in, W1, n_hidden, h1, n_hidden, n_atoms,
                            n_hidden, n_in, 0)));
    bias_silu_kernel<<<512, 256, 0, ctx->stream>>>(h1, b1, n_atoms, n_hidden,
                                                   h1b, pre1);
    LAUNCH_CHECK(ctx);
    TRY((gemm<false, false>(ctx, h1b, n_hidden, W2, n_hidden, h2, n_hidden,
                            n_atoms, n_hidden, n_hidden, 0)));
    bias_silu_kernel<<<512, 256, 0, ctx->stream>>>(h2, b2, n_atoms, n_hidden,
                                                   h2b, pre2);
    LAUNCH_CHECK(ctx);
    head_kernel<<<(n_atoms * 32 + 255) / 256, 256, 0, ctx->stream>>>(
        h2, w3, b3, n_atoms, n_hidden, y);
    LAUNCH_CHECK(ctx);
  }
  reduce_by_config_kernel<<<n_configs, 256, 0, ctx->stream>>>(y, d_off,
                                                              n_configs, energy);
  LAUNCH_CHECK(ctx);
  std::lock_guard<std::mutex> lk(g_mlp_mu);
  MlpState &S = g_mlp[ctx];
  S.n_atoms = n_atoms;
  S.n_in = n_in;
  S.n_hidden = n_hidden;
  S.n_configs = n_configs;
  S.feat = X;
  S.w1 = W1;
  S.w2 = W2;
  S.w3 = w3;
  return PYIID_OK;
}

extern "C" int pyiid_mlp_backward(pyiid_ctx *ctx, const double *d_energy,
                                  float *g_w1, float *g_b1, float *g_w2,
                                  float *g_b2, float *g_w3, float *g_b3) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  MlpState S;
  {
    std::lock_guard<std::mutex> lk(g_mlp_mu);
    auto it = g_mlp.find(ctx);
    if (it == g_mlp.end() || !it->second.feat)
      return fail(ctx, PYIID_ERR_INVALID_ARG,
                  "pyiid_mlp_backward needs a preceding pyiid_mlp_forward");
    S = it->second;
  }
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  const int n = S.n_atoms, H = S.n_hidden, I = S.n_in;
  if (n == 0) {
    CUDA_TRY(ctx, cudaMemsetAsync(g_w1, 0, sizeof(float) * I * H, ctx->stream));
    CUDA_TRY(ctx, cudaMemsetAsync(g_b1, 0, sizeof(float) * H, ctx->stream));
    CUDA_TRY(ctx, cudaMemsetAsync(g_w2, 0, sizeof(float) * H * H, ctx->stream));
    CUDA_TRY(ctx, cudaMemsetAsync(g_b2, 0, sizeof(float) * H, ctx->stream));
    CUDA_TRY(ctx, cudaMemsetAsync(g_w3, 0, sizeof(float) * H, ctx->stream));
    CUDA_TRY(ctx, cudaMemsetAsync(g_b3, 0, sizeof(float), ctx->stream));
    return PYIID_OK;
  }
  const size_t nh = (size_t)n * H;
  void *p;
  TRY(ensure(ctx, "sg_h1b", nh * sizeof(__nv_bfloat16), &p));
  __nv_bfloat16 *h1b = static_cast<__nv_bfloat16 *>(p);
  TRY(ensure(ctx, "sg_pre1", nh * sizeof(float), &p));
  float *pre1 = static_cast<float *>(p);
  TRY(ensure(ctx, "sg_h2", nh * sizeof(float), &p));
  float *h2 = static_cast<float *>(p);
  TRY(ensure(ctx, "sg_pre2", nh * sizeof(float), &p));
  float *pre2 = static_cast<float *>(p);
  TRY(ensure(ctx, "sg_d1", nh * sizeof(float), &p));
  float *d1 = static_cast<float *>(p);
  TRY(ensure(ctx, "sg_d2", nh * sizeof(float), &p));
  float *d2 = static_cast<float *>(p);
  TRY(ensure(ctx, "sg_d1b", nh * sizeof(__nv_bfloat16), &p));
  __nv_bfloat16 *d1b = static_cast<__nv_bfloat16 *>(p);
  TRY(ensure(ctx, "sg_d2b", nh * sizeof(__nv_bfloat16), &p));
  __nv_bfloat16 *d2b = static_cast<__nv_bfloat16 *>(p);
  const int *cfg = g_mlp[ctx].atom_cfg;
  // head: dw3 = sum_a de h2[a], db3 = sum_a de, dh2 = de w3
  column_sum_kernel<<<H, 256, 0, ctx->stream>>>(h2, n, H, d_energy, cfg, g_w3);
  LAUNCH_CHECK(ctx);
  column_sum_kernel<<<1, 256, 0, ctx->stream>>>(nullptr, n, 1, d_energy, cfg,
                                                g_b3);
  LAUNCH_CHECK(ctx);
  head_backward_kernel<<<512, 256, 0, ctx->stream>>>(d_energy, cfg, h2, S.w3,
                                                     n, H, d2, d2b);
  LAUNCH_CHECK(ctx);
  // layer 2: dz2 = dh2 silu'(pre2); dW2 = h1^T dz2; db2 = colsum; dh1 = dz2 W2^T
  silu_backward_kernel<<<512, 256, 0, ctx->stream>>>(d2, pre2, nh, d2b, d2);
  LAUNCH_CHECK(ctx);
  TRY((gemm<true, false>(ctx, h1b, H, d2b, H, g_w2, H, H, H, n, 0)));
  column_sum_kernel<<<H, 256, 0, ctx->stream>>>(d2, n, H, nullptr, nullptr,
                                                g_b2);
  LAUNCH_CHECK(ctx);
  TRY((gemm<false, true>(ctx, d2b, H, S.w2, H, d1, H, n, H, H, 0)));
  // layer 1: dz1 = dh1 silu'(pre1); dW1 = X^T dz1; db1 = colsum
  silu_backward_kernel<<<512, 256, 0, ctx->stream>>>(d1, pre1, nh, d1b, d1);
  LAUNCH_CHECK(ctx);
  TRY((gemm<true, false>(ctx, S.feat, I, d1b, H, g_w1, H, I, H, n, 0)));
  column_sum_kernel<<<H, 256, 0, ctx->stream>>>(d1, n, H, nullptr, nullptr,
                                                g_b1);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

// ======================================================= surrogate forces
// The surrogate's energy and forces for trajectories driven by it (the
// first stage of delayed-acceptance HMC): descriptors from neighbour lists,
// the MLP forward, its gradient with respect to the descriptors (the same
// BF16 tensor-core GEMMs transposed) and the per-atom forces.  Workspace and
// the atom -> configuration map use their own buffers ("sf_*"), so training
// calls on the same context never move what a captured graph of this path
// reads.
namespace {

std::mutex g_sf_mu;
std::unordered_map<const pyiid_ctx *, uint64_t> g_sf_key;

int sf_config_map(pyiid_ctx *ctx, const int32_t *offsets, int n_configs,
                  int **d_cfg, int **d_off) {
  const int total = offsets[n_configs];
  const uint64_t key = fnv1a(offsets, sizeof(int32_t) * (n_configs + 1));
  void *p;
  TRY(ensure(ctx, "sf_cfg", sizeof(int) * std::max(total, 1), &p));
  *d_cfg = static_cast<int *>(p);
  TRY(ensure(ctx, "sf_off", sizeof(int) * (n_configs + 1), &p));
  *d_off = static_cast<int *>(p);
  std::lock_guard<std::mutex> lk(g_sf_mu);
  auto it = g_sf_key.find(ctx);
  // the key mixes the buffer address so a reallocated buffer is refilled
  const uint64_t full = fnv1a(d_cfg, sizeof(*d_cfg), key);
  if (it == g_sf_key.end() || it->second != full) {
    std::vector<int> cfg(std::max(total, 1), 0);
    for (int c = 0; c < n_configs; ++c)
      for (int a = offsets[c]; a < offsets[c + 1]; ++a) cfg[a] = c;
    CUDA_TRY(ctx, cudaMemcpy(*d_cfg, cfg.data(), sizeof(int) * cfg.size(),
                             cudaMemcpyHostToDevice));
    CUDA_TRY(ctx, cudaMemcpy(*d_off, offsets, sizeof(int) * (n_configs + 1),
                             cudaMemcpyHostToDevice));
    g_sf_key[ctx] = full;
  }
  return PYIID_OK;
}

}  // namespace

// the fused MLP kernel's dynamic shared memory exceeds the 48 KB default:
// raise its limit once per device
int fused_mlp_attr(pyiid_ctx *ctx) {
  static std::mutex mu;
  static bool done[64] = {};
  std::lock_guard<std::mutex> lk(mu);
  if (ctx->device >= 0 && ctx->device < 64 && done[ctx->device])
    return PYIID_OK;
  CUDA_TRY(ctx, cudaFuncSetAttribute(mlp_fused_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(FusedMlpSmem)));
  CUDA_TRY(ctx, cudaFuncSetAttribute(mlptc::mlp_tc_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     mlptc::kSmemBytes));
  CUDA_TRY(ctx, cudaFuncSetAttribute(mlptc::mlp_tc2_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     mlptc::kSmemBytes2));
  if (ctx->device >= 0 && ctx->device < 64) done[ctx->device] = true;
  return PYIID_OK;
}

extern "C" int pyiid_neighbor_list(pyiid_ctx *ctx, const float *positions,
                                   const int32_t *offsets, int n_configs,
                                   float r_list, int max_nb, int32_t *nbr_idx,
                                   int32_t *nbr_cnt) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  TRY(check_offsets(ctx, offsets, n_configs));
  if (!(r_list > 0)) return fail(ctx, PYIID_ERR_INVALID_ARG, "r_list <= 0");
  if (max_nb < 1) return fail(ctx, PYIID_ERR_INVALID_ARG, "max_nb < 1");
  const int total = offsets[n_configs];
  if (total == 0) return PYIID_OK;
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  int *d_cfg, *d_off;
  TRY(sf_config_map(ctx, offsets, n_configs, &d_cfg, &d_off));
  const int warps = 8;
  neighbor_list_kernel<<<(total + warps - 1) / warps, 32 * warps, 0,
                         ctx->stream>>>(positions, d_cfg, d_off, total,
                                        r_list * r_list, max_nb, nbr_idx,
                                        nbr_cnt);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}

extern "C" int pyiid_surrogate_forces(
    pyiid_ctx *ctx, const float *positions, const int32_t *offsets,
    int n_configs, const int32_t *nbr_idx, const int32_t *nbr_cnt, int max_nb,
    int n_centres, float r_cut, float sigma, const void *w1_bf16,
    const float *b1, const void *w2_bf16, const float *b2, const float *w3,
    const float *b3, int n_hidden, float scale, double *energy,
    float *forces, void *feat_bf16) {
  if (!ctx) return fail(nullptr, PYIID_ERR_INVALID_ARG, "null context");
  TRY(check_offsets(ctx, offsets, n_configs));
  if (n_centres < 2 || n_centres > 64)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "n_centres must be in [2, 64]");
  if (!(r_cut > 0) || !(sigma > 0))
    return fail(ctx, PYIID_ERR_INVALID_ARG, "r_cut and sigma must be > 0");
  if (n_hidden < 1 || max_nb < 1)
    return fail(ctx, PYIID_ERR_INVALID_ARG, "bad sizes");
  if (forces && n_centres % 8 != 0)
    return fail(ctx, PYIID_ERR_INVALID_ARG,
                "forces need n_centres divisible by 8 (got %d)", n_centres);
  const int n = offsets[n_configs];
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  int *d_cfg, *d_off;
  TRY(sf_config_map(ctx, offsets, n_configs, &d_cfg, &d_off));
  const int H = n_hidden, C = n_centres;
  const size_t nh = (size_t)std::max(n, 1) * H;
  void *p;
  __nv_bfloat16 *X = static_cast<__nv_bfloat16 *>(feat_bf16);
  if (!X) {
    TRY(ensure(ctx, "sf_x", (size_t)std::max(n, 1) * C * sizeof(__nv_bfloat16),
               &p));
    X = static_cast<__nv_bfloat16 *>(p);
  }
  TRY(ensure(ctx, "sf_h1", nh * sizeof(float), &p));
  float *h1 = static_cast<float *>(p);
  TRY(ensure(ctx, "sf_pre1", nh * sizeof(float), &p));
  float *pre1 = static_cast<float *>(p);
  TRY(ensure(ctx, "sf_h1b", nh * sizeof(__nv_bfloat16), &p));
  __nv_bfloat16 *h1b = static_cast<__nv_bfloat16 *>(p);
  TRY(ensure(ctx, "sf_h2", nh * sizeof(float), &p));
  float *h2 = static_cast<float *>(p);
  TRY(ensure(ctx, "sf_pre2", nh * sizeof(float), &p));
  float *pre2 = static_cast<float *>(p);
  TRY(ensure(ctx, "sf_h2b", nh * sizeof(__nv_bfloat16), &p));
  __nv_bfloat16 *h2b = static_cast<__nv_bfloat16 *>(p);
  TRY(ensure(ctx, "sf_y", sizeof(float) * std::max(n, 1), &p));
  float *y = static_cast<float *>(p);
  TRY(ensure(ctx, "sf_gx", (size_t)std::max(n, 1) * C * sizeof(float), &p));
  float *gx = static_cast<float *>(p);
  const __nv_bfloat16 *W1 = static_cast<const __nv_bfloat16 *>(w1_bf16);
  const __nv_bfloat16 *W2 = static_cast<const __nv_bfloat16 *>(w2_bf16);
  const int warps = 8;
  const int wgrid = (std::max(n, 1) + warps - 1) / warps;
  if (n > 0 && C == kFC && H == kFH) {
    // the 32-128-128 net: one fused kernel for y and dE/dfeat
    rbf_features_nl_kernel<<<wgrid, 32 * warps, 0, ctx->stream>>>(
        positions, nbr_idx, nbr_cnt, max_nb, n, C, r_cut, sigma, X, nullptr);
    LAUNCH_CHECK(ctx);
    TRY(fused_mlp_attr(ctx));
    TRY(ensure(ctx, "sf_gh", (size_t)std::max(n, 1) * C * sizeof(__half), &p));
    __half *gh = static_cast<__half *>(p);
    const int tiles = (n + mlptc::kRows - 1) / mlptc::kRows;
    if (ctx->mlp_variant == 1) {
      // tensor-memory MLP: one persistent CTA per SM, 128 atoms per tile
      // (measured 151 us against 70 us for the register-resident kernel on
      // 64,000 atoms: the SiLU epilogues, one thread per row on 4 warps,
      // dominate; kept as a variant)
      mlptc::mlp_tc_kernel<<<std::min(tiles, std::max(1, ctx->n_sms)), 128,
                             mlptc::kSmemBytes, ctx->stream>>>(
          X, n, W1, b1, W2, b2, w3, b3, y, gh, ctx->d_status);
    } else if (ctx->mlp_variant == 2) {
      // two tiles in flight per CTA, two threads per row
      mlptc::mlp_tc2_kernel<<<std::min((tiles + 1) / 2,
                                       std::max(1, ctx->n_sms)),
                              512, mlptc::kSmemBytes2, ctx->stream>>>(
          X, n, W1, b1, W2, b2, w3, b3, y, gh, ctx->d_status);
    } else {
      const int blocks =
          std::min((n + 127) / 128, 2 * std::max(1, ctx->n_sms));
      mlp_fused_kernel<<<blocks, 256, sizeof(FusedMlpSmem), ctx->stream>>>(
          X, n, W1, b1, W2, b2, w3, b3, y, gh);
    }
    LAUNCH_CHECK(ctx);
    reduce_by_config_kernel<<<n_configs, 256, 0, ctx->stream>>>(
        y, d_off, n_configs, energy);
    LAUNCH_CHECK(ctx);
    if (forces) {
      rbf_forces_nl_kernel<__half><<<wgrid, 32 * warps, 0, ctx->stream>>>(
          positions, nbr_idx, nbr_cnt, max_nb, n, C, r_cut, sigma, gh, scale,
          forces);
      LAUNCH_CHECK(ctx);
    }
    return PYIID_OK;
  }
  if (n > 0) {
    rbf_features_nl_kernel<<<wgrid, 32 * warps, 0, ctx->stream>>>(
        positions, nbr_idx, nbr_cnt, max_nb, n, C, r_cut, sigma, X, nullptr);
    LAUNCH_CHECK(ctx);
    TRY((gemm<false, false>(ctx, X, C, W1, H, h1, H, n, H, C, 0)));
    bias_silu_kernel<<<512, 256, 0, ctx->stream>>>(h1, b1, n, H, h1b, pre1);
    LAUNCH_CHECK(ctx);
    TRY((gemm<false, false>(ctx, h1b, H, W2, H, h2, H, n, H, H, 0)));
    bias_silu_kernel<<<512, 256, 0, ctx->stream>>>(h2, b2, n, H, h2b, pre2);
    LAUNCH_CHECK(ctx);
    head_kernel<<<(n * 32 + 255) / 256, 256, 0, ctx->stream>>>(h2, w3, b3, n,
                                                                H, y);
    LAUNCH_CHECK(ctx);
  }
  reduce_by_config_kernel<<<n_configs, 256, 0, ctx->stream>>>(y, d_off,
                                                              n_configs, energy);
  LAUNCH_CHECK(ctx);
  if (!forces || n == 0) return PYIID_OK;
  // dE/dh2 = w3 for every atom; back through both layers to dE/dfeat.
  // h1/h2 and their BF16 copies are dead now: reuse them as gradients.
  broadcast_rows_kernel<<<512, 256, 0, ctx->stream>>>(w3, n, H, h2, h2b);
  LAUNCH_CHECK(ctx);
  silu_backward_kernel<<<512, 256, 0, ctx->stream>>>(h2, pre2, nh, h2b, h2);
  LAUNCH_CHECK(ctx);
  TRY((gemm<false, true>(ctx, h2b, H, W2, H, h1, H, n, H, H, 0)));
  silu_backward_kernel<<<512, 256, 0, ctx->stream>>>(h1, pre1, nh, h1b, h1);
  LAUNCH_CHECK(ctx);
  TRY((gemm<false, true>(ctx, h1b, H, W1, H, gx, C, n, C, H, 0)));
  rbf_forces_nl_kernel<float><<<wgrid, 32 * warps, 0, ctx->stream>>>(
      positions, nbr_idx, nbr_cnt, max_nb, n, C, r_cut, sigma, gx, scale,
      forces);
  LAUNCH_CHECK(ctx);
  return PYIID_OK;
}
