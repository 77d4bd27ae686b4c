// noalloc.cu -- the neighbour-grid sort (compute_particle_bins) for callers
// that cannot allocate device memory.
//
// The store path (create_psdata_cuda) owns its scratch: per-particle arrival
// slots, scan partial sums, the crowded-cell queue and the buffer the
// crowded-cell sort works in, all carved from one cudaMalloc.  Some callers
// cannot make that allocation:
//   - engines and plugin hosts that own all device memory through their
//     own pool and forbid other allocations in their frame loop;
//   - real-time loops where the implicit device synchronisation of
//     cudaMalloc/cudaFree is not acceptable.
// sph_compute_particle_bins_noalloc serves them: the caller passes its own
// device buffers for the inputs and outputs, and the scratch comes from one
// file-scope device array of fixed size, below.  Every GPU that loads this
// library holds that array (about 12.3 MB) until the process exits.
//
// The array is shared by every call on a device and keeps the previous
// call's contents; everything that must start at zero is cleared at the
// start of each call.  Calls that overlap on the GPU (on different streams,
// or from different host threads) race on the array: order them on one
// stream.  The first call on each device looks up the array's device
// address (cudaGetSymbolAddress) with that device current; make that first
// call before any stream capture.  Later calls look the address up again
// whenever their stream is not capturing, so a context that was torn down
// and made again (cudaDeviceReset) gets the array's new address.
#include <mutex>

#include "launch.h"
#include "sph_gb300.h"
#include "sph_internal.h"

namespace {

constexpr unsigned kBlock = 256;
constexpr size_t kMaxParticles = SPH_NOALLOC_MAX_PARTICLES;
constexpr size_t kMaxCells = SPH_NOALLOC_MAX_CELLS;
constexpr size_t kMaxScanTiles = kMaxCells / SPH_SCAN_TILE;
constexpr size_t kMaxBig = kMaxParticles / (SPH_SMALL_CELL + 1) + 2;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Layout of the scratch array (byte offsets).
constexpr size_t kSlot = 0;                                                    // u32[n]
constexpr size_t kSortBuf = kSlot + align256(4 * kMaxParticles);               // u32[2n], crowded-cell sort
constexpr size_t kScan = kSortBuf + align256(8 * kMaxParticles);               // u32[tiles]
constexpr size_t kBig = kScan + align256(4 * kMaxScanTiles);                   // u32[1 + queue]
constexpr size_t kN = kBig + align256(4 * kMaxBig);                            // u32 n
constexpr size_t kStatus = kN + 256;                                           // u32 status
constexpr size_t kDesc = kStatus + 256;                                        // SceneDesc
constexpr size_t kPMap = kDesc + align256(sizeof(SceneDesc));                  // BlockWork per 256 particles
constexpr size_t kCMap = kPMap + align256(sizeof(BlockWork) * (kMaxParticles / kBlock));
constexpr size_t kSMap = kCMap + align256(sizeof(BlockWork) * (kMaxCells / kBlock));
constexpr size_t kBytes = kSMap + align256(sizeof(BlockWork) * kMaxScanTiles);

}  // namespace

// The scratch of every call on this device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

namespace {

std::mutex g_mu;
void *g_base[128];  // device address of g_noalloc_scratch, per device

// Writes the one-scene table, the n counter, a cleared status word and the
// block maps into the scratch array.
__global__ void k_noalloc_setup(unsigned char *base, SceneDesc d, unsigned n) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    if (t == 0) {
        *reinterpret_cast<SceneDesc *>(base + kDesc) = d;
        *reinterpret_cast<unsigned *>(base + kN) = n;
        *reinterpret_cast<unsigned *>(base + kStatus) = 0u;
    }
    BlockWork *pm = reinterpret_cast<BlockWork *>(base + kPMap);
    BlockWork *cm = reinterpret_cast<BlockWork *>(base + kCMap);
    BlockWork *sm = reinterpret_cast<BlockWork *>(base + kSMap);
    const unsigned np = (n + kBlock - 1) / kBlock;
    const unsigned nc = (d.num_cells + kBlock - 1) / kBlock;
    const unsigned ns = (d.num_cells + SPH_SCAN_TILE - 1) / SPH_SCAN_TILE;
    for (unsigned b = t; b < np; b += stride) pm[b] = BlockWork{0u, b * kBlock};
    for (unsigned b = t; b < nc; b += stride) cm[b] = BlockWork{0u, b * kBlock};
    for (unsigned b = t; b < ns; b += stride) sm[b] = BlockWork{0u, b * SPH_SCAN_TILE};
}

// ORs the call's status bits (SphStatus) into the caller's word.
__global__ void k_noalloc_status(const unsigned char *base, unsigned *out) {
    *out |= *reinterpret_cast<const unsigned *>(base + kStatus);
}

}  // namespace

extern "C" int sph_compute_particle_bins_noalloc(const float *position, unsigned int n, const float *gridbounds,
                                                  unsigned int rx, unsigned int ry, unsigned int rz,
                                                  unsigned int *gridcell, unsigned int *gridcount,
                                                  unsigned int *celloffset, unsigned int *cellparticles,
                                                  unsigned int *status, void *stream) {
    const unsigned long long cells = (unsigned long long)rx * ry * rz;
    if (n > kMaxParticles) {
        sph_set_error("sph_compute_particle_bins_noalloc: %u particles exceed the fixed scratch's limit of %zu",
                      n, kMaxParticles);
        return -1;
    }
    if (cells == 0 || cells > kMaxCells) {
        sph_set_error("sph_compute_particle_bins_noalloc: grid %ux%ux%u has %llu cells; the fixed scratch "
                      "allows 1 to %zu",
                      rx, ry, rz, cells, kMaxCells);
        return -1;
    }
    if (!gridbounds || !gridcount || !celloffset || (n && (!position || !gridcell || !cellparticles))) {
        sph_set_error("sph_compute_particle_bins_noalloc: null buffer");
        return -1;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 128) {
        sph_set_error("sph_compute_particle_bins_noalloc: no current device (%s)", cudaGetErrorString(e));
        return -1;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the address is looked up again outside a stream capture (a context
    // made anew after cudaDeviceReset loads the array elsewhere); a
    // capturing stream uses the address its device had last
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(s, &cap);
    if (e != cudaSuccess) {
        sph_set_error("sph_compute_particle_bins_noalloc: stream: %s", cudaGetErrorString(e));
        return -1;
    }
    unsigned char *base;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_base[dev] || cap == cudaStreamCaptureStatusNone) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) {
                sph_set_error("sph_compute_particle_bins_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
                return -1;
            }
            g_base[dev] = p;
        }
        base = static_cast<unsigned char *>(g_base[dev]);
    }
    SceneDesc d{};
    d.n = reinterpret_cast<const unsigned *>(base + kN);
    d.gridbounds = gridbounds;
    d.position = const_cast<float *>(position);
    d.gridcell = gridcell;
    d.gridcount = gridcount;
    d.celloffset = celloffset;
    d.cellparticles = cellparticles;
    d.pnum = n;
    d.gridres[0] = rx;
    d.gridres[1] = ry;
    d.gridres[2] = rz;
    d.num_cells = (unsigned)cells;
    d.programs = PROG_COMMON;
    d.slot = reinterpret_cast<unsigned *>(base + kSlot);
    d.spos = reinterpret_cast<float4 *>(base + kSortBuf);
    d.scan_sums = reinterpret_cast<unsigned *>(base + kScan);
    d.num_scan_blocks = (unsigned)((cells + SPH_SCAN_TILE - 1) / SPH_SCAN_TILE);
    d.big_cells = reinterpret_cast<unsigned *>(base + kBig);
    d.status = reinterpret_cast<unsigned *>(base + kStatus);
    k_noalloc_setup<<<64, 256, 0, s>>>(base, d, n);

    Launch L{};
    L.scenes = reinterpret_cast<const SceneDesc *>(base + kDesc);
    L.num_scenes = 1;
    L.particles = {reinterpret_cast<const BlockWork *>(base + kPMap), (n + kBlock - 1) / kBlock};
    L.cells = {reinterpret_cast<const BlockWork *>(base + kCMap), (unsigned)((cells + kBlock - 1) / kBlock)};
    L.scan = {reinterpret_cast<const BlockWork *>(base + kSMap), d.num_scan_blocks};
    L.pair_particles = L.particles;
    L.block = kBlock;
    L.pair_block = kBlock;
    L.grid_cap = 1u << 30;
    L.stream = s;
    sph_launch_bins(L);
    if (status) k_noalloc_status<<<1, 1, 0, s>>>(base, status);
    e = sph_check_launch("sph_compute_particle_bins_noalloc");
    return e == cudaSuccess ? 0 : -1;
}
