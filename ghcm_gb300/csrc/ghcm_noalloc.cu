// ghcm_solve_device_noalloc: the device solve for callers that cannot
// allocate GPU memory.
//
// Some callers of this library run where a cudaMalloc is not allowed or not
// safe to make: inside a host that owns every device allocation through its
// own pool and forbids foreign ones, in code paths that must not synchronise
// the device (cudaMalloc/cudaFree can), or in long-running services that must
// not grow their footprint after start-up. ghcm_solve_device needs a context
// (ghcm_create allocates its workspace, pinned staging and events); this entry
// point needs none. The scheduler's scratch - per-tile flags, keys and
// smallest times, the two active lists, the job list, the control block and
// the instance record - lives in one file-scope __device__ array below, sized
// for at most GHCM_NOALLOC_MAX_TILES tiles. Every GPU that loads the library
// holds that array (about 7 MiB) until the process exits.
//
// The caller passes the field, seeds and output on the device, as for
// ghcm_solve_device. Calls share the one array: two calls that overlap on the
// GPU (different streams, or different host threads) race on it and give
// wrong results; serialise them. Everything a solve needs zeroed (the control
// block) or initialised (the per-tile state) is set at the start of each call.
// The first call on a device looks the array's device address up with
// cudaGetSymbolAddress (with that device current). Every call reads the
// control block back and synchronises its stream, so none can be captured
// into a CUDA graph.
#include "ghcm_device.cuh"
#include "ghcm_host.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>

namespace ghcm {
namespace {

constexpr size_t kSlot = static_cast<size_t>(GHCM_NOALLOC_MAX_TILES) * sizeof(uint32_t);
constexpr size_t kCtlBytes = 2048;
constexpr size_t kInstBytes = 256;
// flags | key | tmin | list0 | list1 | jobs | epoch | control block | instance
constexpr size_t kScratchBytes = 7 * kSlot + kCtlBytes + kInstBytes;
static_assert(sizeof(Ctl) <= kCtlBytes && sizeof(Inst) <= kInstBytes, "scratch slots too small");

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::atomic<void*> g_scratch_addr[kMaxDevices];
std::mutex g_setup_mutex;

// Device address of g_noalloc_scratch on the current device (looked up once
// per device, with that device current). nullptr on failure.
void* scratch_address(int dev) {
    if (dev < 0 || dev >= kMaxDevices) return nullptr;
    void* p = g_scratch_addr[dev].load(std::memory_order_acquire);
    if (p) return p;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    p = g_scratch_addr[dev].load(std::memory_order_relaxed);
    if (p) return p;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return nullptr;
    }
    g_scratch_addr[dev].store(p, std::memory_order_release);
    return p;
}

__global__ void k_store_inst(Inst* dst, Inst inst) { *dst = inst; }

}  // namespace
}  // namespace ghcm

extern "C" int ghcm_solve_device_noalloc(const ghcm_config* cfg, const float* d_field, int input_is_speed,
                                         uint32_t width, uint32_t height, float h, const uint32_t* d_seeds_xy,
                                         uint32_t n_seeds, float* d_time_out, void* stream) {
    using namespace ghcm;
    int rc = check_config(cfg);
    if (rc != GHCM_OK) return rc;
    if (cfg->schedule != GHCM_SCHEDULE_PLAIN) return GHCM_ERR_BAD_ARG;  // no model without a context
    if (!d_field || !d_time_out || width == 0 || height == 0 || (n_seeds && !d_seeds_xy)) return GHCM_ERR_BAD_ARG;
    if (!(h > 0.f) || !(h < 3.0e38f)) return GHCM_ERR_BAD_ARG;
    uint32_t const B = cfg->block_size;
    // tile counts in 64 bits: (width + B - 1) in 32 bits wraps for widths near 2^32
    uint64_t const tiles64 = ((static_cast<uint64_t>(width) + B - 1) / B) * ((static_cast<uint64_t>(height) + B - 1) / B);
    if (tiles64 > GHCM_NOALLOC_MAX_TILES || width > kMaxSide || height > kMaxSide) return GHCM_ERR_TOO_LARGE;
    uint32_t const tiles = static_cast<uint32_t>(tiles64);

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GHCM_ERR_CUDA;
    if (cfg->device >= 0 && cfg->device != dev) return GHCM_ERR_BAD_ARG;  // runs on the current device
    int sms = 0, coop = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (sms <= 0 || !coop) return GHCM_ERR_UNSUPPORTED;
    LaunchInfo li{};
    if (query_persistent(static_cast<int>(B), cfg->kernel == GHCM_KERNEL_FIM, &li) != 0 || li.blocks_per_sm <= 0)
        return GHCM_ERR_UNSUPPORTED;
    char* base = static_cast<char*>(scratch_address(dev));
    if (!base) return GHCM_ERR_CUDA;

    Sched s;
    std::memset(&s, 0, sizeof(s));
    Inst inst;
    std::memset(&inst, 0, sizeof(inst));
    inst.in = d_field;
    inst.time = d_time_out;
    inst.w = width;
    inst.h = height;
    inst.tiles_x = (width + B - 1) / B;
    inst.tiles_y = (height + B - 1) / B;
    inst.spacing = h;
    inst.in_is_speed = input_is_speed ? 1u : 0u;
    inst.seeds = d_seeds_xy;
    inst.n_seeds = n_seeds;
    inst.cost_cap = cost_cap_of(*cfg);
    bool const aligned = (width % 4u == 0u) && (reinterpret_cast<uintptr_t>(d_field) % 16u == 0u) &&
                         (reinterpret_cast<uintptr_t>(d_time_out) % 16u == 0u);
    EncodeTiledFn const enc = tensor_map_encoder();
    inst.tma = (cfg->use_tma && aligned && encode_tile_map(enc, &s.tmap_time, d_time_out, width, height, B) &&
                encode_tile_map(enc, &s.tmap_in, d_field, width, height, B))
                   ? 1
                   : 0;

    s.flags = reinterpret_cast<uint32_t*>(base + 0 * kSlot);
    s.key = reinterpret_cast<uint32_t*>(base + 1 * kSlot);
    s.tmin = reinterpret_cast<float*>(base + 2 * kSlot);
    s.list[0] = reinterpret_cast<uint32_t*>(base + 3 * kSlot);
    s.list[1] = reinterpret_cast<uint32_t*>(base + 4 * kSlot);
    s.jobs = reinterpret_cast<uint32_t*>(base + 5 * kSlot);
    s.epoch = reinterpret_cast<uint32_t*>(base + 6 * kSlot);
    s.ctl = reinterpret_cast<Ctl*>(base + 7 * kSlot);
    Inst* d_inst = reinterpret_cast<Inst*>(base + 7 * kSlot + kCtlBytes);
    s.insts = d_inst;
    s.tile_inst = nullptr;
    s.num_tiles = tiles;
    s.num_insts = 1;
    fill_sched_params(s, *cfg, sms, tiles);

    cudaStream_t const st = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    k_store_inst<<<1, 1, 0, st>>>(d_inst, inst);
    if ((e = cudaGetLastError()) != cudaSuccess) return GHCM_ERR_CUDA;
    if ((e = cudaMemsetAsync(s.ctl, 0, sizeof(Ctl), st)) != cudaSuccess) return GHCM_ERR_CUDA;
    if ((e = launch_init(s, 1, static_cast<uint64_t>(width) * height, n_seeds, static_cast<int>(B), sms, st)) != cudaSuccess)
        return GHCM_ERR_CUDA;
    LaunchInfo wl{};
    if (wide_for(li, sms, s.max_jobs) &&
        query_persistent(static_cast<int>(B), cfg->kernel == GHCM_KERNEL_FIM, &wl, true) == 0 && wl.blocks_per_sm > 0)
        li = wl;
    if ((e = launch_persistent(static_cast<int>(B), cfg->kernel == GHCM_KERNEL_FIM, s, persistent_grid(li, sms, s.max_jobs), st,
                               li.wide)) !=
        cudaSuccess)
        return GHCM_ERR_CUDA;
    // the whole control block back (error bits, and the failing site id of an
    // index check in GHCM_CHECKED builds)
    Ctl c;
    if ((e = cudaMemcpyAsync(&c, s.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return GHCM_ERR_CUDA;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return GHCM_ERR_CUDA;
    report_checks(c);
    return status_from_error(c.error);
}
