// Allocation-free neighbour pass: the Z-grid see pass of the test model ("agent_see")
// run on positions already in device memory, with every intermediate buffer (keys,
// permutation, radix counts, cell table, reordered positions, accumulators) carved out
// of one fixed array in the library's own device memory instead of cudaMalloc.
//
// For callers that cannot allocate device memory at the point where they need the pass:
// hosts whose memory manager owns the whole device heap (a framework's caching allocator
// or a fixed per-process budget), plugins that may not allocate after initialisation, and
// latency-sensitive loops that cannot afford cudaMalloc's implicit synchronisation.
//
// Limits and sharing rules (also stated in include/tay_gpu.h):
//   * at most kNoallocMaxAgents agents per call; larger calls are rejected with an error;
//   * the grid has at most 64 cells per axis; wider domains get larger cells (results are
//     unchanged, only slower);
//   * the array is shared by every call in the process and keeps the last call's
//     contents; everything that must start at zero is cleared at the start of each call;
//     two calls whose work overlaps on the GPU (different streams, or different host
//     threads) overwrite each other's data and race;
//   * every GPU that loads the library holds the array until the process exits;
//   * every call looks up the array's device address in the current device's context
//     (cudaGetSymbolAddress, a host-side query), so a context that was destroyed and
//     created again (cudaDeviceReset) never leaves a stale address behind;
//   * the call waits for its own work (it synchronises the stream and reads back the
//     device error word), so it may not be called while any stream is capturing;
//   * a CUDA error left pending by earlier, unrelated work is not taken over: the call
//     refuses to start and leaves that error in place for its owner.
#include <cstdio>

#include "model.cuh"
#include "tay_gpu.h"

namespace tgpu {
namespace {

constexpr uint32_t kNoallocMaxAgents = 65536;
constexpr uint32_t kNoallocAxisCells = 64;
constexpr uint32_t kNoallocTable = kNoallocAxisCells * kNoallocAxisCells * kNoallocAxisCells;
constexpr uint32_t kNoallocTiles = kNoallocMaxAgents / kSortTile;
constexpr uint32_t kNoallocCtas = kNoallocMaxAgents / kSeeThreads;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// byte offsets inside the scratch array
constexpr size_t kOffSpec = 0;
constexpr size_t kOffBox = align256(kOffSpec + sizeof(SegmentSpec));
constexpr size_t kOffGrid = align256(kOffBox + sizeof(BoxAcc));
constexpr size_t kOffPairs = align256(kOffGrid + sizeof(SegGrid));
constexpr size_t kOffTileSeg = align256(kOffPairs + sizeof(unsigned long long));
constexpr size_t kOffRadii = align256(kOffTileSeg + sizeof(uint32_t) * kNoallocTiles);
constexpr size_t kOffCtx = align256(kOffRadii + sizeof(float4));
constexpr size_t kOffCta = align256(kOffCtx + sizeof(float4));
constexpr size_t kOffKeys0 = align256(kOffCta + sizeof(uint2) * kNoallocCtas);
constexpr size_t kOffKeys1 = align256(kOffKeys0 + sizeof(uint32_t) * kNoallocMaxAgents);
constexpr size_t kOffVals0 = align256(kOffKeys1 + sizeof(uint32_t) * kNoallocMaxAgents);
constexpr size_t kOffVals1 = align256(kOffVals0 + sizeof(uint32_t) * kNoallocMaxAgents);
constexpr size_t kOffSortScratch = align256(kOffVals1 + sizeof(uint32_t) * kNoallocMaxAgents);
constexpr size_t kOffErr = align256(kOffSortScratch + sort_scratch_bytes(1, kNoallocTiles));
constexpr size_t kOffTable = align256(kOffErr + sizeof(uint32_t));
constexpr size_t kOffPos = align256(kOffTable + sizeof(uint2) * kNoallocTable);
constexpr size_t kOffAcc = align256(kOffPos + sizeof(float4) * kNoallocMaxAgents);
constexpr size_t kNoallocBytes = align256(kOffAcc + sizeof(float4) * kNoallocMaxAgents);
static_assert(kNoallocBytes < (8u << 20), "scratch stays modest");

}  // namespace

// The scratch array: device memory reserved when the library is loaded.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

namespace {

// Writes the one-segment description, the tile and CTA tables, the radii and context,
// and clears the pair counter, the accumulators and the cell table.
__global__ void noalloc_setup_kernel(unsigned char *scratch, SegmentSpec spec, float4 radii, uint32_t n) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t threads = gridDim.x * blockDim.x;
    if (tid == 0) {
        *reinterpret_cast<SegmentSpec *>(scratch + kOffSpec) = spec;
        *reinterpret_cast<unsigned long long *>(scratch + kOffPairs) = 0ull;
        *reinterpret_cast<float4 *>(scratch + kOffRadii) = radii;
        *reinterpret_cast<float4 *>(scratch + kOffCtx) = radii;
    }
    uint32_t *tile_seg = reinterpret_cast<uint32_t *>(scratch + kOffTileSeg);
    for (uint32_t t = tid; t < spec.tile_count; t += threads) tile_seg[t] = 0u;
    uint2 *cta = reinterpret_cast<uint2 *>(scratch + kOffCta);
    const uint32_t ctas = (n + kSeeThreads - 1) / kSeeThreads;
    for (uint32_t c = tid; c < ctas; c += threads) cta[c] = make_uint2(0u, c * kSeeThreads);
    float4 *acc = reinterpret_cast<float4 *>(scratch + kOffAcc);
    for (uint32_t i = tid; i < n; i += threads) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    uint2 *table = reinterpret_cast<uint2 *>(scratch + kOffTable);
    for (uint32_t c = tid; c < kNoallocTable; c += threads) table[c] = make_uint2(0u, 0u);
}

// Results back in the caller's order: out[perm[i]] = acc[i].
__global__ void noalloc_unpermute_kernel(const uint32_t *perm, const float4 *acc, float4 *out, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[perm[i]] = acc[i];
}

thread_local char g_noalloc_err[256];

int noalloc_fail(int code, const char *msg) {
    snprintf(g_noalloc_err, sizeof(g_noalloc_err), "%s", msg);
    return code;
}

}  // namespace
}  // namespace tgpu

using namespace tgpu;

extern "C" unsigned tgpu_noalloc_max_agents(void) { return kNoallocMaxAgents; }

extern "C" const char *tgpu_noalloc_last_error(void) { return g_noalloc_err; }

extern "C" int tgpu_see_noalloc(const float *positions, unsigned n, const float *radii, const float *min_part_sizes,
                                float *out, void *stream) {
    if (n > kNoallocMaxAgents) {
        char msg[160];
        snprintf(msg, sizeof(msg), "tgpu_see_noalloc: %u agents exceed the maximum of %u", n, kNoallocMaxAgents);
        return noalloc_fail(TGPU_ERR_ARG, msg);
    }
    if (n == 0) return TGPU_OK;
    if (!positions || !out || !radii || !min_part_sizes)
        return noalloc_fail(TGPU_ERR_ARG, "tgpu_see_noalloc: null pointer argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

    // an error pending from earlier work would be indistinguishable from this call's own
    // launch errors below: leave it to its owner and do nothing
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        char msg[200];
        snprintf(msg, sizeof(msg), "tgpu_see_noalloc: an earlier CUDA error is pending (%s); not started",
                 cudaGetErrorString(e));
        return noalloc_fail(TGPU_ERR_CUDA, msg);
    }
    // the array's device address in the current context, looked up on every call
    void *scratch_addr = nullptr;
    e = cudaGetSymbolAddress(&scratch_addr, g_noalloc_scratch);
    if (e != cudaSuccess) {
        cudaGetLastError();  // the failed lookup's own error
        char msg[200];
        snprintf(msg, sizeof(msg), "tgpu_see_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return noalloc_fail(TGPU_ERR_CUDA, msg);
    }
    unsigned char *scratch = static_cast<unsigned char *>(scratch_addr);

    SegmentSpec spec{};
    spec.begin = 0;
    spec.count = n;
    spec.table_base = 0;
    spec.table_cap = kNoallocTable;
    spec.tile_begin = 0;
    spec.tile_count = (n + kSortTile - 1) / kSortTile;
    spec.axis_cells_max = kNoallocAxisCells;
    spec.fixed_box = 0;
    for (int a = 0; a < 3; ++a) {
        spec.part[a] = min_part_sizes[a] > 0.0f ? min_part_sizes[a] : 1.0f;
        spec.reach[a] = radii[a];
    }
    const float4 r4 = make_float4(radii[0], radii[1], radii[2], radii[3]);
    noalloc_setup_kernel<<<152, 256, 0, st>>>(scratch, spec, r4, n);

    SortLaunch L{};
    L.specs = reinterpret_cast<const SegmentSpec *>(scratch + kOffSpec);
    L.tile_seg = reinterpret_cast<const uint32_t *>(scratch + kOffTileSeg);
    L.box = reinterpret_cast<BoxAcc *>(scratch + kOffBox);
    L.grids = reinterpret_cast<SegGrid *>(scratch + kOffGrid);
    L.pos = reinterpret_cast<const float4 *>(positions);
    L.keys[0] = reinterpret_cast<uint32_t *>(scratch + kOffKeys0);
    L.keys[1] = reinterpret_cast<uint32_t *>(scratch + kOffKeys1);
    L.vals[0] = reinterpret_cast<uint32_t *>(scratch + kOffVals0);
    L.vals[1] = reinterpret_cast<uint32_t *>(scratch + kOffVals1);
    L.sort_scratch = reinterpret_cast<uint32_t *>(scratch + kOffSortScratch);
    L.err = reinterpret_cast<uint32_t *>(scratch + kOffErr);
    L.table = reinterpret_cast<uint2 *>(scratch + kOffTable);
    L.segments = 1;
    L.tiles = spec.tile_count;
    L.key_bits = 18;  // 6 bits per axis for 64 cells

    launch_box(L, st);
    uint32_t *skeys = nullptr, *perm = nullptr;
    launch_sort(L, st, &skeys, &perm);
    float4 *pos_sorted = reinterpret_cast<float4 *>(scratch + kOffPos);
    GatherSet gs{};
    gs.src_f4[0] = L.pos;
    gs.dst_f4[0] = pos_sorted;
    gs.nf4 = 1;
    launch_cell_table(L, skeys, 1, st, perm, &gs);  // and the positions into cell order

    // the test model's see pass (agent_see alone): accumulators into the acc array
    const KernelDesc &k = model_test_basic()->kernels[0];
    float4 *acc = reinterpret_cast<float4 *>(scratch + kOffAcc);
    SeeLaunch S{};
    S.specs = L.specs;
    S.box = L.box;
    S.grids = L.grids;
    S.table = L.table;
    S.cta_table = reinterpret_cast<const uint2 *>(scratch + kOffCta);
    S.radii = reinterpret_cast<const float4 *>(scratch + kOffRadii);
    S.ctx = reinterpret_cast<const char *>(scratch + kOffCtx);
    S.ctx_stride = sizeof(float4);
    S.act_ctx = S.ctx;
    S.act_ctx_stride = sizeof(float4);
    S.ctas = (n + kSeeThreads - 1) / kSeeThreads;
    S.skip_self = 1;
    S.stage_cap = 0;
    S.stage_cells = 0;
    S.union_factor = 1;
    S.pairs = reinterpret_cast<unsigned long long *>(scratch + kOffPairs);
    S.telemetry = nullptr;
    for (int c = 0; c < 4; ++c) {
        S.io.in_f4[c] = c == 0 ? pos_sorted : acc;
        S.io.out_f4[c] = c == 0 ? pos_sorted : acc;
    }
    k.launch_see(S, 0, st);
    noalloc_unpermute_kernel<<<(n + 255) / 256, 256, 0, st>>>(perm, acc, reinterpret_cast<float4 *>(out), n);
    launch_cell_table(L, skeys, 0, st);
    // launch errors first (only this call's: nothing was pending at entry), then the
    // errors of the work itself
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        char msg[200];
        snprintf(msg, sizeof(msg), "tgpu_see_noalloc: %s", cudaGetErrorString(e));
        return noalloc_fail(TGPU_ERR_CUDA, msg);
    }
    uint32_t err = 0;
    e = cudaMemcpy(&err, scratch + kOffErr, sizeof(err), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && err) {
        cudaMemset(scratch + kOffErr, 0, sizeof(err));
        return noalloc_fail(TGPU_ERR_DEVICE, "tgpu_see_noalloc: radix sort look-back wait ran out");
    }
    return TGPU_OK;
}
