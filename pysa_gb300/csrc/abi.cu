// abi.cu -- extern "C" entry points of libpysa_gb (declared in
// include/pysa_gb.h).  Host code only: argument checks, the work list of the
// sweep kernel, variant dispatch and launches on the caller's stream.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ais_api.h"
#include "csr_api.h"
#include "tc_api.h"
#include "wide_api.h"
#include "aux.cuh"
#include "plain_variants.h"
#include "sweep_plain.cuh"

namespace pysa_gb {

extern const PlainVariant kPlainSmall[4];
extern const PlainVariant kPlainLarge[4];

const PlainVariant& plain_variant(int v) {
  return v < 4 ? kPlainSmall[v] : kPlainLarge[v - 4];
}

int plain_variant_for(int n) {
  for (int v = 0; v < kNumPlainVariants; ++v)
    if (n <= 32 * plain_variant(v).nc) return v;
  return -1;
}

static int row_floats(int v) {
  const int nc = plain_variant(v).nc;
  const int ls = nc < 4 ? 4 : (((nc / 4) & 1) ? nc : nc + 4);
  return 32 * ls;
}

static int lane_stride(int v) { return row_floats(v) / 32; }

PlainItemPlan make_item_plan() {
  PlainItemPlan plan;
  for (int v = 0; v < kNumPlainVariants; ++v) {
    const PlainVariant& pv = plain_variant(v);
    plan.nc[v] = pv.nc;
    plan.cpb[v] = pv.gw * pv.w;
    plan.row_floats[v] = row_floats(v);
    plan.start[v] = 0;
  }
  return plan;
}

static thread_local std::string g_last_error;
static unsigned long long* g_tc_trace = nullptr;  // diagnostics, see below
static uint64_t g_unit_wait_ns = 0;  // diagnostics: 0 = the default bound
static int32_t g_decision_mode = 0;   // tensor-core sweep: 0 auto, 1, 2
static int32_t g_round_limit = 12;    // mode 0: block rounds up to this
static int32_t g_tc_max_ctas = 0;     // tensor-core launches: 0 = SM count

static int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int pysa_gb_internal_fail(int code, const char* msg) {
  return fail(code, msg);
}

static int cuda_fail(cudaError_t e, const char* where) {
  return fail(PYSA_GB_ERR_CUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

// Default for the most sweeps one fused tensor-core launch covers.
constexpr int kMaxFusedSweeps = 128;

// Streaming multiprocessors of the current device (cached per device).
static inline bool is_sparse(const pysa_gb_host_tables* h, int i) {
  return h && h->sparse && h->sparse[i];
}

static int sm_count() {
  static int cache[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 1;
  if (cache[dev] == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = v > 0 ? v : 1;
  }
  return cache[dev];
}

// Per-device, per-variant launch geometry, filled on first use.
struct VariantInfo {
  bool ready[2] = {false, false};
  int blocks_per_sm[2] = {0, 0};
};
static VariantInfo g_vinfo[64][kNumPlainVariants];

static int prepare_variant(int v, bool random, int* grid_cap) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev >= 64) return fail(PYSA_GB_ERR_ARG, "device index >= 64");
  VariantInfo& vi = g_vinfo[dev][v];
  const PlainVariant& pv = plain_variant(v);
  if (!vi.ready[random]) {
    const size_t sm = pv.smem(random);
    e = cudaFuncSetAttribute(pv.func(random),
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sm);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
    int bps = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, pv.func(random),
                                                      pv.w * 32, sm);
    if (e != cudaSuccess) return cuda_fail(e, "occupancy query");
    if (bps < 1) return fail(PYSA_GB_ERR_SIZE, "sweep kernel does not fit");
    vi.blocks_per_sm[random] = bps;
    vi.ready[random] = true;
  }
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(e, "SM count");
  *grid_cap = sms * vi.blocks_per_sm[random];
  return PYSA_GB_OK;
}

}  // namespace pysa_gb

using namespace pysa_gb;

extern "C" {

int pysa_gb_abi_version(void) { return PYSA_GB_ABI_VERSION; }

int pysa_gb_set_unit_wait_limit(uint64_t ns) {
  g_unit_wait_ns = ns;
  return PYSA_GB_OK;
}

int pysa_gb_set_decision_mode(int32_t mode) {
  if (mode < 0 || mode > 2)
    return fail(PYSA_GB_ERR_ARG, "decision mode must be 0, 1 or 2");
  g_decision_mode = mode;
  return PYSA_GB_OK;
}

int pysa_gb_set_block_round_limit(int32_t flips) {
  if (flips < 0 || flips > 64)
    return fail(PYSA_GB_ERR_ARG, "block round limit must be in 0..64");
  g_round_limit = flips;
  return PYSA_GB_OK;
}

int pysa_gb_set_tc_max_ctas(int32_t ctas) {
  if (ctas < 0) return fail(PYSA_GB_ERR_ARG, "max CTAs must be >= 0");
  g_tc_max_ctas = ctas;
  return PYSA_GB_OK;
}

int pysa_gb_tc_wrap_piece(int32_t items, int32_t sweeps, int32_t ctas,
                          int32_t share, int32_t piece, int32_t out[3]) {
  if (!out || items < 1 || sweeps < 1 || ctas < 1 || ctas > items ||
      share < 0 || share >= ctas || piece < 0)
    return fail(PYSA_GB_ERR_ARG, "wrap piece: bad arguments");
  int it = -1, sb = 0, sl = 0;
  if (!wrap_piece(items, sweeps, ctas, share, piece, &it, &sb, &sl)) return 0;
  out[0] = it;
  out[1] = sb;
  out[2] = sl;
  return 1;
}

int pysa_gb_set_trace(void* device_buffer) {
  g_tc_trace = reinterpret_cast<unsigned long long*>(device_buffer);
  return PYSA_GB_OK;
}

const char* pysa_gb_last_error(void) { return g_last_error.c_str(); }

int pysa_gb_workspace_bytes(int32_t num_instances,
                            const pysa_gb_host_tables* host, int64_t out[3]) {
  if (num_instances < 0 || !out ||
      (num_instances > 0 &&
       (!host || !host->n || !host->replicas || !host->reads)))
    return fail(PYSA_GB_ERR_ARG, "workspace_bytes: null argument");
  const int32_t* n_host = host ? host->n : nullptr;
  const int32_t* replicas_host = host ? host->replicas : nullptr;
  const int32_t* reads_host = host ? host->reads : nullptr;
  int64_t packed = 0, items = 0;
  int max_nc = 1;
  for (int i = 0; i < num_instances; ++i) {
    const int n = n_host[i];
    if (n < 1) return fail(PYSA_GB_ERR_ARG, "instance with n < 1");
    if (n > PYSA_GB_MAX_N)
      return fail(PYSA_GB_ERR_SIZE, "n exceeds PYSA_GB_MAX_N");
    if (replicas_host[i] < 1 || replicas_host[i] > kMaxReplicas)
      return fail(PYSA_GB_ERR_SIZE, "replicas must be in [1, 512]");
    if (reads_host[i] < 0) return fail(PYSA_GB_ERR_ARG, "negative reads");
    const int64_t chains = (int64_t)replicas_host[i] * reads_host[i];
    if (is_sparse(host, i)) {  // sparse-row sweep: fields only for prepare
      items += (chains + 31) / 32;  // items of 32 chains at the smallest
      const int nc = (n + 31) / 32;
      if (nc > max_nc) max_nc = nc;
      continue;
    }
    if (n > kPlainMaxN) {  // wide-instance sweep: J read in place
      items += (chains + kWideWarps - 1) / kWideWarps;
      const int nc = (n + 31) / 32;
      if (nc > max_nc) max_nc = nc;
      continue;
    }
    const int v = plain_variant_for(n);
    const PlainVariant& pv = plain_variant(v);
    packed += (int64_t)n * row_floats(v);
    const int cpb = pv.gw * pv.w;
    items += (chains + cpb - 1) / cpb;
    if (pv.nc > max_nc) max_nc = pv.nc;
  }
  out[0] = packed;
  out[1] = items * (int64_t)(sizeof(SweepItem) / sizeof(int32_t));
  out[2] = 32 * max_nc;
  return (int)items;
}

int pysa_gb_setup(const pysa_gb_problems* p, const pysa_gb_host_tables* host,
                  pysa_gb_workspace* ws, void* stream) {
  if (!p || !ws || !host || !host->n || !host->replicas || !host->reads ||
      !host->chain_off || !host->j_off || !host->ld)
    return fail(PYSA_GB_ERR_ARG, "setup: null argument");
  const int32_t* n_host = host->n;
  const int32_t* replicas_host = host->replicas;
  const int32_t* reads_host = host->reads;
  const int64_t* chain_off_host = host->chain_off;
  int64_t need[3];
  const int items_n = pysa_gb_workspace_bytes(p->num_instances, host, need);
  if (items_n < 0) return items_n;
  if (!ws->packed_j || ws->packed_j_elems < need[0])
    return fail(PYSA_GB_ERR_ARG, "packed_j too small");
  if (!ws->items || ws->num_items < items_n)
    return fail(PYSA_GB_ERR_ARG, "items too small");
  if (ws->field_ld < need[2] || ws->field_ld % 4 != 0)
    return fail(PYSA_GB_ERR_ARG, "field_ld too small or not a multiple of 4");
  if (reinterpret_cast<uintptr_t>(ws->fields) % 16 != 0)
    return fail(PYSA_GB_ERR_ARG, "fields must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  // work list ordered by variant; host-side ranges stored in the workspace
  std::vector<SweepItem> items;
  items.reserve(items_n);
  std::vector<int64_t> poff(p->num_instances);
  int64_t off = 0;
  auto is_wide = [&](int i) {
    return !is_sparse(host, i) && n_host[i] > kPlainMaxN;
  };
  for (int i = 0; i < p->num_instances; ++i) {
    poff[i] = off;
    if (!is_sparse(host, i) && !is_wide(i))
      off += (int64_t)n_host[i] * row_floats(plain_variant_for(n_host[i]));
  }
  for (int v = 0; v < kNumPlainVariants; ++v) {
    ws->variant_start[v] = (int32_t)items.size();
    const PlainVariant& pv = plain_variant(v);
    const int cpb = pv.gw * pv.w;
    for (int i = 0; i < p->num_instances; ++i) {
      if (is_sparse(host, i) || plain_variant_for(n_host[i]) != v) continue;
      const int64_t chains = (int64_t)replicas_host[i] * reads_host[i];
      for (int64_t c = 0; c < chains; c += cpb) {
        SweepItem it;
        it.inst = i;
        it.chain0 = (int32_t)(chain_off_host[i] + c);
        it.nchains = (int32_t)((chains - c) < cpb ? (chains - c) : cpb);
        it.variant = v;
        it.poff_lo = (int32_t)(uint32_t)(poff[i] & 0xffffffffll);
        it.poff_hi = (int32_t)(poff[i] >> 32);
        it.pad0 = it.pad1 = 0;
        items.push_back(it);
      }
    }
    ws->variant_count[v] = (int32_t)items.size() - ws->variant_start[v];
  }
  // sparse instances: up to 128 chains per item of the sparse-row sweep,
  // fewer while the items would leave SMs idle
  ws->csr_item_start = (int32_t)items.size();
  int cpb = kCsrChains;
  {
    int64_t sparse_chains = 0;
    for (int i = 0; i < p->num_instances; ++i)
      if (is_sparse(host, i))
        sparse_chains += (int64_t)replicas_host[i] * reads_host[i];
    const int sms = sm_count();
    while (cpb > 32 && (sparse_chains + cpb - 1) / cpb < sms) cpb /= 2;
  }
  // the sparse-row sweep keeps every chain's spin words (and, in random
  // order, the visiting order and a record slab) in shared memory
  {
    const size_t words = (size_t)(p->max_n + 31) / 32;
    auto smem = [&](int ch) {
      return words * ch * 4 + (size_t)p->max_n * 4 + 17408 + 1024;
    };
    bool any_sparse = false;
    for (int i = 0; i < p->num_instances; ++i)
      any_sparse |= is_sparse(host, i);
    while (cpb > 32 && smem(cpb) > 232448) cpb /= 2;
    if (any_sparse && smem(cpb) > 232448)
      return fail(PYSA_GB_ERR_SIZE,
                  "sparse instances: n too large for the sparse-row sweep's "
                  "shared memory at 32 chains per CTA");
  }
  ws->csr_chains = cpb;
  for (int i = 0; i < p->num_instances; ++i) {
    if (!is_sparse(host, i)) continue;
    if (!p->csr_row_off || !p->csr_ent_off || !p->csr_col || !p->csr_val ||
        (ws->csr_width == 0 && !p->csr_rows))
      return fail(PYSA_GB_ERR_ARG, "sparse instance without csr tables");
    if (ws->csr_width != 0 && ws->csr_width != 4 && ws->csr_width != 8 &&
        ws->csr_width != 16 && ws->csr_width != 32)
      return fail(PYSA_GB_ERR_ARG, "csr_width must be 0, 4, 8, 16 or 32");
    const int64_t chains = (int64_t)replicas_host[i] * reads_host[i];
    for (int64_t c = 0; c < chains; c += cpb) {
      SweepItem it;
      it.inst = i;
      it.chain0 = (int32_t)(chain_off_host[i] + c);
      it.nchains = (int32_t)((chains - c) < cpb ? (chains - c) : cpb);
      it.variant = -1;
      it.poff_lo = it.poff_hi = 0;
      it.pad0 = it.pad1 = 0;
      items.push_back(it);
    }
  }
  ws->csr_item_count = (int32_t)items.size() - ws->csr_item_start;
  // wide dense instances: kWideWarps chains per item; J is read in place
  // with 16-byte loads
  ws->wide_item_start = (int32_t)items.size();
  for (int i = 0; i < p->num_instances; ++i) {
    if (!is_wide(i)) continue;
    if (host->j_off[i] % 4 != 0 || host->ld[i] % 4 != 0 ||
        reinterpret_cast<uintptr_t>(p->J) % 16 != 0)
      return fail(PYSA_GB_ERR_ARG,
                  "instances with n > 4096 need j_off and ld multiples of 4 "
                  "and J 16-byte aligned");
    const int64_t chains = (int64_t)replicas_host[i] * reads_host[i];
    for (int64_t c = 0; c < chains; c += kWideWarps) {
      SweepItem it;
      it.inst = i;
      it.chain0 = (int32_t)(chain_off_host[i] + c);
      it.nchains = (int32_t)((chains - c) < kWideWarps ? (chains - c)
                                                       : kWideWarps);
      it.variant = -2;
      it.poff_lo = it.poff_hi = 0;
      it.pad0 = it.pad1 = 0;
      items.push_back(it);
    }
  }
  ws->wide_item_count = (int32_t)items.size() - ws->wide_item_start;
  if (!items.empty()) {
    cudaError_t e = cudaMemcpyAsync(ws->items, items.data(),
                                    items.size() * sizeof(SweepItem),
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy work list");
  }
  // couplings into the packed row layout, per instance
  for (int i = 0; i < p->num_instances; ++i) {
    if (host->ld[i] < n_host[i])
      return fail(PYSA_GB_ERR_ARG, "ld < n");
    if (is_sparse(host, i) || is_wide(i)) continue;
    const int v = plain_variant_for(n_host[i]);
    launch_pack_rows(p->J + host->j_off[i], host->ld[i], n_host[i],
                     plain_variant(v).nc, lane_stride(v),
                     ws->packed_j + poff[i], st);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "pack couplings");
  return PYSA_GB_OK;
}

static inline bool tc_selected(const pysa_gb_host_tables* host, int i,
                               int min_n) {
  const int n = host->n[i];
  return !is_sparse(host, i) && n >= (min_n < 64 ? 64 : min_n) && n <= 2048;
}

// Chains per tensor-core work item of every selected instance.  fixed = 0:
// a CTA's full tensor memory (128/F chains), halved while the batch would
// fill fewer CTAs than the GPU has SMs and the halves still hold whole reads
// (or whole warps when R does not divide 128/F).  fixed > 0: the largest
// multiple of the instance's granule (R, or 32) not above min(fixed, 128/F),
// at least one granule.  fixed < 0: one granule (the smallest items, for
// sizing).  0 for instances left to the plain kernel.
static std::vector<int> tc_item_sizes(int num_instances,
                                      const pysa_gb_host_tables* host,
                                      int min_n, int fixed) {
  std::vector<int> size(num_instances, 0), gran(num_instances, 32);
  for (int i = 0; i < num_instances; ++i) {
    if (!tc_selected(host, i, min_n)) continue;
    size[i] = tc_chains_per_cta(host->n[i]);
    if (size[i] % host->replicas[i] == 0) gran[i] = host->replicas[i];
    if (gran[i] > size[i]) gran[i] = size[i];
    if (fixed < 0) {
      size[i] = gran[i];
    } else if (fixed > 0) {
      const int cap = fixed < size[i] ? fixed : size[i];
      const int m = cap / gran[i] * gran[i];
      size[i] = m > 0 ? m : gran[i];
    }
  }
  if (fixed != 0) return size;
  const int sms = sm_count();
  for (;;) {
    int64_t items = 0;
    bool can = false;
    for (int i = 0; i < num_instances; ++i) {
      if (!size[i]) continue;
      const int64_t chains = (int64_t)host->replicas[i] * host->reads[i];
      items += (chains + size[i] - 1) / size[i];
      const int h = size[i] / 2;
      can |= h >= gran[i] && h % gran[i] == 0;
    }
    if (items >= sms || !can) break;
    for (int i = 0; i < num_instances; ++i) {
      const int h = size[i] / 2;
      if (size[i] && h >= gran[i] && h % gran[i] == 0) size[i] = h;
    }
  }
  return size;
}

int pysa_gb_tc_workspace(int32_t num_instances,
                         const pysa_gb_host_tables* host, int32_t terms,
                         int32_t min_n, int64_t out[3]) {
  if (num_instances < 0 || !out || (terms != 1 && terms != 2) ||
      (num_instances > 0 && (!host || !host->n || !host->replicas ||
                             !host->reads)))
    return fail(PYSA_GB_ERR_ARG, "tc_workspace: bad argument");
  for (int i = 0; i < num_instances; ++i)
    if (host->replicas[i] < 1 || host->reads[i] < 0)
      return fail(PYSA_GB_ERR_ARG, "tc_workspace: bad replicas or reads");
  // capacity for the smallest items tc_item_chains can ask for
  const std::vector<int> isz = tc_item_sizes(num_instances, host, min_n, -1);
  int64_t b = 0, d = 0, items = 0;
  for (int i = 0; i < num_instances; ++i) {
    const int n = host->n[i];
    if (!tc_selected(host, i, min_n)) continue;
    b += tc_b_elems(n, terms);
    d += tc_diag_elems(n);
    const int64_t chains = (int64_t)host->replicas[i] * host->reads[i];
    items += (chains + isz[i] - 1) / isz[i];
  }
  out[0] = b;
  out[1] = d;
  out[2] = items * (int64_t)(sizeof(TcItem) / sizeof(int32_t));
  return (int)items;
}

int pysa_gb_tc_setup(const pysa_gb_problems* p, const pysa_gb_host_tables* host,
                     pysa_gb_workspace* ws, void* stream) {
  if (!p || !host || !ws || !host->chain_off || !host->j_off || !host->ld)
    return fail(PYSA_GB_ERR_ARG, "tc_setup: null argument");
  int64_t need[3];
  const int min_n = ws->tc_min_n;
  const int items_n = pysa_gb_tc_workspace(p->num_instances, host,
                                           ws->tc_terms, min_n, need);
  if (items_n < 0) return items_n;
  if (!ws->tc_b || ws->tc_b_elems < need[0] || !ws->tc_diag ||
      ws->tc_diag_elems < need[1] || !ws->tc_items ||
      ws->tc_num_items < items_n || !ws->tc_inst || !ws->tc_sched)
    return fail(PYSA_GB_ERR_ARG, "tc workspace too small");
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<int64_t> boff(p->num_instances), doff(p->num_instances);
  std::vector<int32_t> flags(p->num_instances, 0);
  const PlainItemPlan plan = make_item_plan();
  int64_t bo = 0, dd = 0;
  int live = 0, fusable = 1;
  for (int i = 0; i < p->num_instances; ++i) {
    boff[i] = bo;
    doff[i] = dd;
    if (!tc_selected(host, i, min_n)) {
      if (!is_sparse(host, i) && host->n[i] <= kPlainMaxN)
        live |= 1 << plan.variant_of(host->n[i]);
      continue;
    }
    if (tc_chains_per_cta(host->n[i]) % host->replicas[i] != 0) fusable = 0;
    flags[i] = 1;
    bo += tc_b_elems(host->n[i], ws->tc_terms);
    dd += tc_diag_elems(host->n[i]);
  }
  std::vector<TcItem> items;
  if (ws->tc_item_chains < 0)
    return fail(PYSA_GB_ERR_ARG, "tc_item_chains must be >= 0");
  if (ws->tc_fp8 && ws->tc_terms != 1)
    return fail(PYSA_GB_ERR_ARG, "tc_fp8 needs tc_terms = 1");
  const std::vector<int> isz =
      tc_item_sizes(p->num_instances, host, min_n, ws->tc_item_chains);
  const int folds[3] = {1, 2, 4};
  int uniform = 0;
  for (int v = 0; v < 3; ++v) {
    ws->tc_variant_start[v] = (int32_t)items.size();
    for (int i = 0; i < p->num_instances; ++i) {
      if (!flags[i] || tc_fold_for(host->n[i]) != folds[v]) continue;
      const int64_t chains = (int64_t)host->replicas[i] * host->reads[i];
      const int cc = isz[i];
      for (int64_t c = 0; c < chains; c += cc) {
        TcItem it;
        it.inst = i;
        it.chain0 = (int32_t)(host->chain_off[i] + c);
        it.nchains = (int32_t)((chains - c) < cc ? (chains - c) : cc);
        it.fold = folds[v];
        it.b_off = boff[i];
        it.diag_off = doff[i];
        items.push_back(it);
      }
    }
    ws->tc_variant_count[v] = (int32_t)items.size() - ws->tc_variant_start[v];
    bool same = true;
    for (int k = ws->tc_variant_start[v] + 1; k < (int)items.size(); ++k)
      same = same && host->n[items[k].inst] ==
                         host->n[items[ws->tc_variant_start[v]].inst];
    if (same) uniform |= 1 << v;
  }
  if (!items.empty()) {
    cudaError_t e = cudaMemcpyAsync(ws->tc_items, items.data(),
                                    items.size() * sizeof(TcItem),
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy tc work list");
  }
  if (p->num_instances > 0) {
    cudaError_t e = cudaMemcpyAsync(ws->tc_inst, flags.data(),
                                    flags.size() * sizeof(int32_t),
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy tc instance flags");
  }
  for (int i = 0; i < p->num_instances; ++i) {
    if (!flags[i]) continue;
    cudaError_t e = launch_pack_tc(p->J + host->j_off[i], host->ld[i],
                                   host->n[i], ws->tc_terms, ws->tc_fp8 != 0,
                                   ws->tc_b + boff[i],
                                   ws->tc_diag + doff[i], st);
    if (e != cudaSuccess) return cuda_fail(e, "pack tc tiles");
  }
  if (ws->tc_inst_off && p->num_instances > 0) {
    std::vector<int64_t> off(2 * (size_t)p->num_instances, -1);
    for (int i = 0; i < p->num_instances; ++i)
      if (flags[i]) {
        off[2 * i] = boff[i];
        off[2 * i + 1] = doff[i];
      }
    cudaError_t e = cudaMemcpyAsync(ws->tc_inst_off, off.data(),
                                    off.size() * sizeof(int64_t),
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy tc instance offsets");
  }
  // host vectors above are pageable: the copies are complete on return
  ws->plain_live = live;
  ws->tc_fusable = fusable;
  ws->tc_uniform = uniform;
  ws->tc_enabled = 1;
  return PYSA_GB_OK;
}

int pysa_gb_prepare(const pysa_gb_problems* p, pysa_gb_state* s,
                    pysa_gb_workspace* ws, int32_t set_energies,
                    int32_t init_best, int32_t best_global, void* stream) {
  if (!p || !s || !ws || !ws->fields)
    return fail(PYSA_GB_ERR_ARG, "prepare: null argument");
  PrepArgs a;
  a.p = *p;
  a.s = *s;
  a.fields = ws->fields;
  a.field_ld = ws->field_ld;
  a.set_energies = set_energies;
  a.init_best = init_best;
  a.best_global = best_global;
  launch_prepare(a, (cudaStream_t)stream);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "prepare");
  return PYSA_GB_OK;
}

// Sweeps per work unit for a fused launch of `chunk` sweeps over `items`
// work items: a divisor of chunk between 4 and 16 with the shortest
// estimated launch.  A unit costs its sweeps plus about 0.2 of a sweep to
// move the fields between HBM and tensor memory (measured on the 1024-spin
// QUBO workload: 8-sweep units 195 us per sweep, 1-sweep units 228); the
// launch takes as many unit times as the waves of units over the SMs, and
// at least the units of one item (they run one after another).  Without
// such a divisor, `pref` (the rest goes to the next launch).  128 sweeps
// over 256 items give 8, 20 sweeps give 5 (one launch instead of 16 + 4),
// 128 sweeps of a single item 16.
static int tc_unit_for(int chunk, int pref, int items, int sms) {
  if (chunk <= pref) return chunk;
  double best = 0.0;
  int pick = 0;
  for (int ku = 4; ku <= 16; ++ku) {
    if (chunk % ku) continue;
    const int64_t per_item = chunk / ku;
    const int64_t units = (int64_t)items * per_item;
    int64_t waves = (units + sms - 1) / sms;
    if (waves < per_item) waves = per_item;
    const double cost = (double)waves * (ku + 0.2);
    if (pick == 0 || cost < best - 1e-9) {
      best = cost;
      pick = ku;
    }
  }
  return pick ? pick : pref;
}

int pysa_gb_sweeps(const pysa_gb_problems* p, pysa_gb_state* s,
                   pysa_gb_workspace* ws, const pysa_gb_options* o,
                   int32_t num_sweeps, void* stream) {
  if (!p || !s || !ws || !o)
    return fail(PYSA_GB_ERR_ARG, "sweeps: null argument");
  if (num_sweeps < 0) return fail(PYSA_GB_ERR_ARG, "negative sweep count");
  const bool random = o->update == PYSA_GB_RANDOM;
  if (random && (!ws->perm || ws->perm_slots < 1))
    return fail(PYSA_GB_ERR_ARG, "random order needs a perm workspace");
  if (o->log_omega_stride > 0 && !s->log_omega)
    return fail(PYSA_GB_ERR_ARG, "log_omega buffer missing");
  if (ws->field_ld % 4 != 0 || reinterpret_cast<uintptr_t>(ws->fields) % 16)
    return fail(PYSA_GB_ERR_ARG,
                "fields: row stride must be a multiple of 4 floats and the "
                "base 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  int caps[kNumPlainVariants];
  // random order on the tensor cores needs the repacked-tile slots and as
  // many visiting-order slots
  const bool rand_tc = random && ws->tc_rand_slots > 0 && ws->tc_b_rand &&
                       ws->tc_diag_rand && ws->tc_inst_off &&
                       ws->perm_slots >= ws->tc_rand_slots;
  const bool tc_path = ws->tc_enabled && ws->tc_items && (!random || rand_tc);
  // plain variants that run: all of them, or (tensor-core path) those with
  // instances left to the plain kernel
  const int plain_mask = tc_path ? ws->plain_live : 0xFF;
  for (int v = 0; v < kNumPlainVariants; ++v) {
    caps[v] = 0;
    if (ws->variant_count[v] > 0 && ((plain_mask >> v) & 1)) {
      const int rc = prepare_variant(v, random, &caps[v]);
      if (rc != PYSA_GB_OK) return rc;
    }
  }
  PlainArgs a;
  a.p = *p;
  a.s = *s;
  a.packed_j = ws->packed_j;
  a.perm = ws->perm;
  a.fields = ws->fields;
  a.field_ld = ws->field_ld;
  a.perm_slots = ws->perm_slots > 0 ? ws->perm_slots : 1;
  a.update = o->update;
  a.seed = o->seed;
  a.skip_inst = tc_path ? ws->tc_inst : nullptr;
  XArgs x;
  x.p = *p;
  x.s = *s;
  x.seed = o->seed;
  x.use_pt = o->use_pt;
  x.log_omega_stride = o->log_omega_stride;
  x.exchange_every = o->exchange_every;
  x.pad_ = 0;
  PermArgs pa;
  pa.p = *p;
  pa.sweep_counter = s->sweep_counter;
  pa.perm = ws->perm;
  pa.perm_slots = a.perm_slots;
  pa.seed = o->seed;
  const int phases = o->phases ? o->phases : 3;
  const bool use_tc = tc_path;
  TcArgs ta;
  ta.p = *p;
  ta.s = *s;
  ta.fields = ws->fields;
  ta.field_ld = ws->field_ld;
  ta.terms = ws->tc_terms;
  ta.tc_b = ws->tc_b;
  ta.tc_diag = ws->tc_diag;
  ta.seed = o->seed;
  ta.recompute_every = o->recompute_every;
  ta.use_pt = o->use_pt;
  ta.exchange_every = o->exchange_every;
  ta.unit_wait_ns = g_unit_wait_ns;
  ta.decision_mode = g_decision_mode;
  ta.round_limit = g_round_limit;
  ta.wrap = 0;
  ta.e8 = ws->tc_fp8 != 0;
  ta.sched = ws->tc_sched;
  ta.perm = ws->perm;
  ta.perm_slots = a.perm_slots;
  ta.rand_slots = ws->tc_rand_slots;
  ta.rand_b = ws->tc_b_rand;
  ta.rand_diag = ws->tc_diag_rand;
  ta.rand_b_stride = ws->tc_b_elems;
  ta.rand_diag_stride = ws->tc_diag_elems;
  ta.trace = g_tc_trace;
  const int sms = g_tc_max_ctas > 0 && g_tc_max_ctas < sm_count()
                      ? g_tc_max_ctas
                      : sm_count();
  const int folds[3] = {1, 2, 4};
  int last_v = -1;
  for (int v = 0; v < 3; ++v)
    if (ws->tc_variant_count[v] > 0) last_v = v;
  // Fused launches over items of one size split the launch's item-sweeps
  // evenly over the CTAs (wrap-around units) unless the caller fixed the
  // unit length.
  auto wraps = [&](int v, int fuse) {
    return fuse && ws->tc_unit_sweeps == 0 && ((ws->tc_uniform >> v) & 1);
  };
  // one persistent tensor-core launch per fold: `units` work units of
  // `ku` sweeps per item (or wrap-around units over ku * units sweeps),
  // exchange fused or not
  auto tc_launches = [&](int ku, int units, int fuse) -> int {
    for (int v = 0; v < 3; ++v) {
      const int count = ws->tc_variant_count[v];
      if (count == 0) continue;
      cudaError_t e = cudaMemsetAsync(ws->tc_sched, 0,
                                      sizeof(int32_t) * (2 + (size_t)count), st);
      if (e != cudaSuccess) return cuda_fail(e, "tc schedule reset");
      ta.items = reinterpret_cast<const TcItem*>(ws->tc_items) +
                 ws->tc_variant_start[v];
      ta.num_items = count;
      ta.wrap = wraps(v, fuse) ? 1 : 0;
      ta.unit_sweeps = ta.wrap ? ku * units : ku;
      ta.units_per_item = ta.wrap ? 1 : units;
      ta.fuse_exchange = fuse;
      ta.advance_counter = fuse && v == last_v;
      e = launch_tc(ta, folds[v], random, sms, st);
      if (e != cudaSuccess) return cuda_fail(e, "tc sweep launch");
    }
    return PYSA_GB_OK;
  };
  // Fused: every instance on the tensor cores, exchange inside the kernel
  // (or none), no log-omega; several sweeps per launch with the fields
  // resident in tensor memory.
  const bool fused = use_tc && phases == 3 && ws->plain_live == 0 &&
                     ws->csr_item_count == 0 && ws->wide_item_count == 0 &&
                     o->log_omega_stride == 0 &&
                     (!o->use_pt || ws->tc_fusable) && ws->tc_sched;
  // random order on the tensor cores: visiting orders of the next `cnt`
  // sweeps, and the tiles repacked in those orders
  auto rand_prepare = [&](int cnt) -> int {
    launch_perm(pa, st, cnt);
    cudaError_t e = launch_repack_tc(
        *p, ws->tc_terms, ws->tc_inst_off, ws->perm, a.perm_slots,
        s->sweep_counter, cnt, ws->tc_rand_slots, ws->tc_b_rand,
        ws->tc_b_elems, ws->tc_diag_rand, ws->tc_diag_elems, st);
    return e == cudaSuccess ? PYSA_GB_OK : cuda_fail(e, "tc repack");
  };
  if (fused) {
    const int ku_pref = ws->tc_unit_sweeps > 0 ? ws->tc_unit_sweeps : 8;
    int per_launch =
        ws->tc_launch_sweeps > 0 ? ws->tc_launch_sweeps : kMaxFusedSweeps;
    if (random && per_launch > ws->tc_rand_slots)
      per_launch = ws->tc_rand_slots;
    // items of the largest fold: its launch sets the number of unit waves
    int items = 1;
    bool all_wrap = true;
    for (int v = 0; v < 3; ++v) {
      if (ws->tc_variant_count[v] > items) items = ws->tc_variant_count[v];
      if (ws->tc_variant_count[v] > 0 && !wraps(v, 1)) all_wrap = false;
    }
    int remaining = num_sweeps;
    while (remaining > 0) {
      int chunk = remaining < per_launch ? remaining : per_launch;
      const int ku = ws->tc_unit_sweeps > 0
                         ? (chunk < ku_pref ? chunk : ku_pref)
                     : all_wrap ? chunk
                                : tc_unit_for(chunk, ku_pref, items, sms);
      chunk = chunk / ku * ku;
      if (random) {
        const int rc = rand_prepare(chunk);
        if (rc != PYSA_GB_OK) return rc;
      }
      const int rc = tc_launches(ku, chunk / ku, 1);
      if (rc != PYSA_GB_OK) return rc;
      remaining -= chunk;
    }
    return PYSA_GB_OK;
  }
  for (int sw = 0; sw < num_sweeps; ++sw) {
    if (use_tc && (phases & 1)) {
      if (random) {
        const int rc = rand_prepare(1);
        if (rc != PYSA_GB_OK) return rc;
      }
      const int rc = tc_launches(1, 1, 0);
      if (rc != PYSA_GB_OK) return rc;
    }
    for (int v = 0; (phases & 1) && v < kNumPlainVariants; ++v) {
      if (v == 0 && random) launch_perm(pa, st);
      const int count = ws->variant_count[v];
      if (count == 0 || !((plain_mask >> v) & 1)) continue;
      a.items = reinterpret_cast<const SweepItem*>(ws->items) +
                ws->variant_start[v];
      a.num_items = count;
      const int grid = count < caps[v] ? count : caps[v];
      cudaError_t e = plain_variant(v).launch(a, random, grid, st);
      if (e != cudaSuccess) return cuda_fail(e, "sweep launch");
    }
    if ((phases & 1) && ws->csr_item_count > 0) {
      CsrArgs ca;
      ca.p = *p;
      ca.s = *s;
      ca.perm = ws->perm;
      ca.perm_slots = a.perm_slots;
      ca.num_items = ws->csr_item_count;
      ca.items = reinterpret_cast<const SweepItem*>(ws->items) +
                 ws->csr_item_start;
      ca.seed = o->seed;
      ca.width = ws->csr_width;
      ca.chains = ws->csr_chains > 0 ? ws->csr_chains : kCsrChains;
      cudaError_t e = launch_csr(ca, random, st);
      if (e != cudaSuccess) return cuda_fail(e, "sparse sweep launch");
    }
    if ((phases & 1) && ws->wide_item_count > 0) {
      // (random order: the visiting order was made in the loop above)
      WideArgs wa;
      wa.p = *p;
      wa.s = *s;
      wa.perm = ws->perm;
      wa.fields = ws->fields;
      wa.field_ld = ws->field_ld;
      wa.perm_slots = a.perm_slots;
      wa.items = reinterpret_cast<const SweepItem*>(ws->items) +
                 ws->wide_item_start;
      wa.num_items = ws->wide_item_count;
      wa.pad_ = 0;
      wa.seed = o->seed;
      cudaError_t e = launch_wide(wa, random, 4 * sms, st);
      if (e != cudaSuccess) return cuda_fail(e, "wide sweep launch");
    }
    if (phases & 2) launch_exchange(x, st);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "exchange launch");
  return PYSA_GB_OK;
}

int pysa_gb_energy64(int32_t problem_type, int32_t n, int32_t ld64,
                     const double* J64, const double* h64,
                     const uint32_t* spins, int32_t words, int64_t count,
                     double* out, void* stream) {
  if (!J64 || !h64 || !spins || !out || n < 1 || ld64 < n || count < 0 ||
      words < (n + 31) / 32)
    return fail(PYSA_GB_ERR_ARG, "energy64: bad argument");
  launch_energy64(problem_type, n, ld64, J64, h64, spins, words, count, out,
                  (cudaStream_t)stream);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "energy64");
  return PYSA_GB_OK;
}

int pysa_gb_unpack(int32_t problem_type, int32_t n, const uint32_t* spins,
                   int32_t words, int64_t count, float* out, int32_t out_ld,
                   void* stream) {
  if (!spins || !out || n < 1 || out_ld < n || count < 0 ||
      words < (n + 31) / 32)
    return fail(PYSA_GB_ERR_ARG, "unpack: bad argument");
  launch_unpack(problem_type, n, spins, words, count, out, out_ld,
                (cudaStream_t)stream);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "unpack");
  return PYSA_GB_OK;
}

int pysa_gb_energy64_tables(const pysa_gb_problems* p,
                            const pysa_gb_host_tables* host, int32_t inst,
                            const uint32_t* spins, int32_t words,
                            int64_t count, double* out, void* stream) {
  if (!p || !host || !spins || !out || inst < 0 ||
      inst >= p->num_instances || count < 0)
    return fail(PYSA_GB_ERR_ARG, "energy64_tables: bad argument");
  if (words < (host->n[inst] + 31) / 32)
    return fail(PYSA_GB_ERR_ARG, "energy64_tables: words too small");
  launch_energy64_tables(*p, inst, spins, words, count, out,
                         (cudaStream_t)stream);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "energy64_tables");
  return PYSA_GB_OK;
}

int pysa_gb_pack(int32_t problem_type, int32_t n, const float* x,
                 int32_t x_ld, int64_t count, uint32_t* spins, int32_t words,
                 void* stream) {
  if (!x || !spins || n < 1 || x_ld < n || count < 0 ||
      words < (n + 31) / 32)
    return fail(PYSA_GB_ERR_ARG, "pack: bad argument");
  launch_pack(problem_type, n, x, x_ld, count, spins, words,
              (cudaStream_t)stream);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "pack");
  return PYSA_GB_OK;
}

int pysa_gb_load_problem(const pysa_gb_problems* p,
                         const pysa_gb_host_tables* host, int32_t inst,
                         const float* P, int32_t p_ld, void* stream) {
  if (!p || !host || !P || inst < 0 || inst >= p->num_instances)
    return fail(PYSA_GB_ERR_ARG, "load_problem: bad argument");
  const int n = host->n[inst], ld = host->ld[inst];
  if (n < 1 || p_ld < n || ld < n)
    return fail(PYSA_GB_ERR_ARG, "load_problem: bad sizes");
  if (is_sparse(host, inst))
    return fail(PYSA_GB_ERR_ARG,
                "load_problem: dense problems only (a sparse instance keeps "
                "no dense couplings)");
  launch_load_problem(*p, inst, n, ld, P, p_ld, (cudaStream_t)stream);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "load_problem");
  return PYSA_GB_OK;
}

int pysa_gb_ais(const pysa_gb_problems* p, pysa_gb_state* s,
                pysa_gb_workspace* ws, const pysa_gb_ais_options* o,
                const float* temps, double* log_w, void* stream) {
  if (!p || !s || !ws || !o || !temps || !log_w || !ws->fields)
    return fail(PYSA_GB_ERR_ARG, "ais: null argument");
  if (p->num_instances < 1)
    return fail(PYSA_GB_ERR_ARG, "ais: no instance");
  if (p->max_n > 1024) return fail(PYSA_GB_ERR_SIZE, "ais: n > 1024");
  if (o->num_temps < 0) return fail(PYSA_GB_ERR_ARG, "ais: num_temps < 0");
  if (o->update == PYSA_GB_RANDOM &&
      (!ws->perm || ws->perm_slots < o->num_temps))
    return fail(PYSA_GB_ERR_ARG, "ais: perm workspace needs num_temps slots");
  if (o->reference == 1 && !(o->p > 0.0 && o->p < 1.0))
    return fail(PYSA_GB_ERR_ARG, "ais: bernoulli p must be in (0, 1)");
  if (o->max_samples < 0) return fail(PYSA_GB_ERR_ARG, "ais: max_samples < 0");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (o->update == PYSA_GB_RANDOM) {
    e = launch_perm_all(p->n, p->num_instances, p->max_n, o->num_temps,
                        o->seed, ws->perm, st);
    if (e != cudaSuccess) return cuda_fail(e, "ais: orders");
  }
  AisArgs a;
  a.problem_type = p->problem_type;
  a.words = p->words;
  a.num_temps = o->num_temps;
  a.update = o->update;
  a.ref = o->reference;
  a.order = o->order;
  a.max_n = p->max_n;
  a.num_instances = p->num_instances;
  a.p = o->p;
  a.seed = o->seed;
  a.n_tab = p->n;
  a.ld_tab = p->ld;
  a.replicas = p->replicas;
  a.reads = p->reads;
  a.j_off = p->j_off;
  a.chain_off = p->chain_off;
  a.J = p->J;
  a.temps = temps;
  a.perm = ws->perm;
  a.fields = ws->fields;
  a.field_ld = ws->field_ld;
  a.pad_ = 0;
  a.spins = s->spins;
  a.energies = s->energies;
  a.log_w = log_w;
  a.status = s->status;
  const int64_t max_samples =
      o->max_samples > 0 ? o->max_samples : p->num_chains;
  if (max_samples > 0) {
    e = launch_ais(a, max_samples, st);
    if (e != cudaSuccess) return cuda_fail(e, "ais launch");
  }
  return PYSA_GB_OK;
}

static const int kLogzChunkBits = 12;

int64_t pysa_gb_logz_parts(int32_t num_instances, int32_t max_n) {
  if (num_instances < 0 || max_n < 1 || max_n > 34) return -1;
  const int B = max_n < kLogzChunkBits ? max_n : kLogzChunkBits;
  const int64_t threads = (int64_t)1 << (max_n - B);
  return (int64_t)num_instances * ((threads + 255) / 256);
}

int pysa_gb_logz_exact(const pysa_gb_problems* p, double beta,
                       double* part_max, double* part_sum, void* stream) {
  if (!p || !part_max || !part_sum)
    return fail(PYSA_GB_ERR_ARG, "logz: null argument");
  if (p->max_n < 1 || p->max_n > 34)
    return fail(PYSA_GB_ERR_SIZE, "logz: n must be in [1, 34]");
  LogzArgs a;
  a.problem_type = p->problem_type;
  a.num_instances = p->num_instances;
  a.chunk_bits = kLogzChunkBits;
  a.beta = beta;
  a.n = p->n;
  a.ld = p->ld;
  a.j_off = p->j_off;
  a.h_off = p->h_off;
  a.J = p->J;
  a.h = p->h;
  a.part_max = part_max;
  a.part_sum = part_sum;
  cudaError_t e = launch_logz(a, p->max_n, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "logz launch");
  return PYSA_GB_OK;
}

}  // extern "C"
