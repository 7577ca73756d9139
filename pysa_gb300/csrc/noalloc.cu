// noalloc.cu -- allocation-free variant of the plain PT sweep entry point.
//
// Some callers cannot allocate device memory at all: a plugin running inside
// a host application whose CUDA memory is entirely owned by the host's own
// pool, a real-time loop where cudaMalloc's implicit device synchronisation
// is not acceptable, or C code with no device allocator of its own.  For them
// pysa_gb_sweeps_noalloc takes only the inputs and outputs (problems and
// chain state) and keeps every scratch array of the sweep -- local fields,
// visiting orders, packed couplings and the work list -- in one file-scope
// device array of fixed size, kNoAllocScratchBytes.
//
// Properties a caller must know:
//   * Every GPU that loads this library holds kNoAllocScratchBytes of device
//     memory for the array until the process exits.
//   * All calls share the array and it keeps the last call's contents; the
//     entry point rebuilds everything it reads from it on every call.  Calls
//     that overlap on the GPU (on different streams, or from different host
//     threads without ordering) race on the array.
//   * The first call on each device resolves the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture.  The address is cached for the life of the
//     process: cudaDeviceReset (or anything else that re-creates the
//     device's primary context) leaves it stale, so do not call this entry
//     point again on a device after resetting it.
//   * Dense couplings of at most 4096 spins per instance (the
//     register-resident plain kernel): a batch with a sparse-row instance
//     (pysa_gb_host_tables.sparse) or a wider one is rejected before
//     anything is enqueued.
//   * It allocates nothing: no cudaMalloc / cudaFree, no host heap.  The
//     work list is rebuilt on the device on every call by one CTA in
//     O(instances / 256 + log 256) steps.
#include <mutex>

#include "aux.cuh"
#include "plain_variants.h"
#include "sweep_plain.cuh"
#include "wide_api.h"

namespace pysa_gb {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;  // 64 MiB

static __device__ __align__(256) unsigned char
    g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mutex;
static void* g_noalloc_ptr[64] = {};

// Device address of the scratch array for the current device (host code
// cannot use the symbol itself: it names a host-side stand-in).
static int noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) return PYSA_GB_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return PYSA_GB_ERR_CUDA;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return PYSA_GB_OK;
}

// Work list on the device, built by one CTA: thread t owns a contiguous
// segment of instances; the segments' item counts (per kernel variant) and
// packed-coupling sizes are scanned across the CTA in shared memory, then
// every thread writes its segment's items from those starts.
constexpr int kItemThreads = 256;

__global__ void __launch_bounds__(kItemThreads)
    k_noalloc_items(const int32_t* n, const int32_t* replicas,
                    const int32_t* reads, const int64_t* chain_off,
                    int num_instances, PlainItemPlan plan, SweepItem* items) {
  constexpr int NV = kNumPlainVariants;
  __shared__ int64_t s_sum[NV + 1][kItemThreads];  // items per variant, floats
  const int t = threadIdx.x;
  const int per = (num_instances + kItemThreads - 1) / kItemThreads;
  const int i0 = min(t * per, num_instances);
  const int i1 = min(i0 + per, num_instances);
  auto items_of = [&](int i, int v) {
    return ((int64_t)replicas[i] * reads[i] + plan.cpb[v] - 1) / plan.cpb[v];
  };
  for (int v = 0; v <= NV; ++v) s_sum[v][t] = 0;
  for (int i = i0; i < i1; ++i) {
    const int v = plan.variant_of(n[i]);
    s_sum[v][t] += items_of(i, v);
    s_sum[NV][t] += (int64_t)n[i] * plan.row_floats[v];
  }
  __syncthreads();
  for (int off = 1; off < kItemThreads; off <<= 1) {  // inclusive scans
    int64_t add[NV + 1];
#pragma unroll
    for (int v = 0; v <= NV; ++v) add[v] = t >= off ? s_sum[v][t - off] : 0;
    __syncthreads();
#pragma unroll
    for (int v = 0; v <= NV; ++v) s_sum[v][t] += add[v];
    __syncthreads();
  }
  int64_t pos[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v)
    pos[v] = plan.start[v] + (t > 0 ? s_sum[v][t - 1] : 0);
  int64_t poff = t > 0 ? s_sum[NV][t - 1] : 0;
  for (int i = i0; i < i1; ++i) {
    const int v = plan.variant_of(n[i]);
    const int64_t chains = (int64_t)replicas[i] * reads[i];
    int64_t p = 0;
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (k == v) p = pos[k];
    for (int64_t c = 0; c < chains; c += plan.cpb[v], ++p) {
      SweepItem it;
      it.inst = i;
      it.chain0 = (int32_t)(chain_off[i] + c);
      it.nchains = (int32_t)((chains - c) < plan.cpb[v] ? (chains - c)
                                                         : plan.cpb[v]);
      it.variant = v;
      it.poff_lo = (int32_t)(uint32_t)(poff & 0xffffffffll);
      it.poff_hi = (int32_t)(poff >> 32);
      it.pad0 = it.pad1 = 0;
      items[p] = it;
    }
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (k == v) pos[k] = p;
    poff += (int64_t)n[i] * plan.row_floats[v];
  }
}

}  // namespace pysa_gb

using namespace pysa_gb;

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

extern "C" int pysa_gb_sweeps_noalloc(const pysa_gb_problems* p,
                                      pysa_gb_state* s,
                                      const pysa_gb_host_tables* host,
                                      const pysa_gb_options* o, int32_t init,
                                      int32_t num_sweeps, void* stream) {
  if (!p || !s || !host || !o || !host->n || !host->replicas || !host->reads ||
      !host->chain_off || !host->j_off || !host->ld)
    return pysa_gb_internal_fail(PYSA_GB_ERR_ARG,
                                 "sweeps_noalloc: null argument");
  // dense couplings only: the sizes below have no room for the sparse-row
  // kernel's layout, so such a batch is refused before anything is enqueued
  if (host->sparse)
    for (int i = 0; i < p->num_instances; ++i)
      if (host->sparse[i])
        return pysa_gb_internal_fail(
            PYSA_GB_ERR_ARG,
            "sweeps_noalloc: sparse-row instances are not supported (dense "
            "couplings only); use pysa_gb_sweeps with a workspace");
  // the register-resident plain kernel only (n <= 4096)
  for (int i = 0; i < p->num_instances; ++i)
    if (host->n[i] > kPlainMaxN)
      return pysa_gb_internal_fail(
          PYSA_GB_ERR_SIZE,
          "sweeps_noalloc: instances with more than 4096 spins are not "
          "supported; use pysa_gb_sweeps with a workspace");
  int64_t need[3];
  const int items_n = pysa_gb_workspace_bytes(p->num_instances, host, need);
  if (items_n < 0) return items_n;
  // scratch layout: fields | visiting orders (1 slot) | packed J | work list
  const size_t fields_b = align256((size_t)p->num_chains * need[2] * 4);
  const size_t perm_b =
      align256((size_t)p->num_instances * (size_t)p->max_n * 4);
  const size_t packed_b = align256((size_t)need[0] * 4);
  const size_t items_b = align256((size_t)items_n * sizeof(SweepItem));
  const size_t total = fields_b + perm_b + packed_b + items_b;
  if (total > kNoAllocScratchBytes)
    return pysa_gb_internal_fail(
        PYSA_GB_ERR_SIZE,
        "sweeps_noalloc: this batch needs more scratch than the fixed "
        "64 MiB array (fields + orders + packed couplings + work list); "
        "use pysa_gb_sweeps with a caller-allocated workspace");
  void* base = nullptr;
  if (noalloc_scratch(&base) != PYSA_GB_OK)
    return pysa_gb_internal_fail(PYSA_GB_ERR_CUDA,
                                 "sweeps_noalloc: cudaGetSymbolAddress failed");
  unsigned char* b = static_cast<unsigned char*>(base);
  pysa_gb_workspace ws = {};
  ws.fields = reinterpret_cast<float*>(b);
  ws.field_ld = (int32_t)need[2];
  ws.perm = reinterpret_cast<int32_t*>(b + fields_b);
  ws.perm_slots = 1;
  ws.packed_j = reinterpret_cast<float*>(b + fields_b + perm_b);
  ws.packed_j_elems = need[0];
  ws.items = reinterpret_cast<int32_t*>(b + fields_b + perm_b + packed_b);
  ws.num_items = items_n;
  ws.tc_enabled = 0;
  cudaStream_t st = (cudaStream_t)stream;

  // work list (device-built) and host-side ranges per kernel variant
  PlainItemPlan plan = make_item_plan();
  for (int v = 0; v < kNumPlainVariants; ++v) plan.start[v] = 0;
  int32_t counts[kNumPlainVariants] = {};
  for (int i = 0; i < p->num_instances; ++i) {
    const int v = plain_variant_for(host->n[i]);
    counts[v] += (int32_t)(((int64_t)host->replicas[i] * host->reads[i] +
                            plan.cpb[v] - 1) / plan.cpb[v]);
  }
  int32_t acc = 0;
  for (int v = 0; v < kNumPlainVariants; ++v) {
    plan.start[v] = acc;
    ws.variant_start[v] = acc;
    ws.variant_count[v] = counts[v];
    acc += counts[v];
  }
  if (p->num_instances > 0) {
    k_noalloc_items<<<1, kItemThreads, 0, st>>>(
        p->n, p->replicas, p->reads, p->chain_off, p->num_instances, plan,
        reinterpret_cast<SweepItem*>(ws.items));
  }
  int64_t poff = 0;
  for (int i = 0; i < p->num_instances; ++i) {
    const int v = plain_variant_for(host->n[i]);
    if (host->ld[i] < host->n[i])
      return pysa_gb_internal_fail(PYSA_GB_ERR_ARG, "sweeps_noalloc: ld < n");
    launch_pack_rows(p->J + host->j_off[i], host->ld[i], host->n[i],
                     plain_variant(v).nc, plan.row_floats[v] / 32,
                     ws.packed_j + poff, st);
    poff += (int64_t)host->n[i] * plan.row_floats[v];
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return pysa_gb_internal_fail(PYSA_GB_ERR_CUDA,
                                 "sweeps_noalloc: set-up launch failed");
  // local fields from the spins on every call (the array may hold another
  // call's data); energies and best_* only when starting fresh
  int rc = pysa_gb_prepare(p, s, &ws, init ? 1 : 0, init ? 1 : 0,
                           o->best_global, stream);
  if (rc != PYSA_GB_OK) return rc;
  return pysa_gb_sweeps(p, s, &ws, o, num_sweeps, stream);
}
