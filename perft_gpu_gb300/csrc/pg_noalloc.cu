// pg_noalloc.cu -- batched perft for callers that must not allocate device
// memory.
//
// Some callers cannot call cudaMalloc: a serving process that reserved all of
// the GPU's memory up front for its own pool, a framework whose allocator
// owns the device and forbids side allocations, or code that runs where
// allocation is not allowed (a host callback, a timed region that must not
// call into the allocator).  pg_perft_batch_noalloc serves them: every byte
// of working memory it needs lives in one file-scope device array of a fixed
// size (NA_SCRATCH_BYTES, 60 MiB), which every GPU that loads the library
// holds until the process exits.  The caller passes device pointers for the
// inputs and the output; nothing is allocated by the call (no cudaMalloc,
// cudaFree or allocating library routine).  The call synchronises its stream
// (it reads the partition and the children totals back to the host) and
// returns when d_out is written.
//
// The kernels are the engine's own (root partition, leaf, count, scan,
// expand), launched with the scratch array instead of engine-owned buffers,
// for depths 0..3: a depth-3 root is expanded once into the scratch level and
// both levels finish in the two-ply leaf kernel.  Every size check (positions,
// depths, the children of the depth-3 positions of both sides together) is
// made before the first leaf kernel, so a call that returns PG_ERR_CAPACITY
// has only zeroed d_out.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "pg_kernels.cuh"

namespace pg {
namespace {

constexpr u32 NA_MAX_ROOTS = 1u << 16;      // positions per call
constexpr u32 NA_MAX_CHILDREN = 1u << 20;   // depth-2 nodes made from depth-3 roots per call (both sides)
constexpr int NA_MAX_DEPTH = 3;
constexpr int NA_T = 256;

constexpr u64 align256(u64 x) { return (x + 255) & ~255ull; }
// scratch layout
constexpr u64 NA_L0_PL = 0;                                               // 3 planes x 64 Ki x 16 B
constexpr u64 NA_L0_GRP = align256(NA_L0_PL + 3ull * NA_MAX_ROOTS * 16);
constexpr u64 NA_L0_REM = align256(NA_L0_GRP + 4ull * NA_MAX_ROOTS);
constexpr u64 NA_L0_CNT = align256(NA_L0_REM + 1ull * NA_MAX_ROOTS);
constexpr u64 NA_L0_OFFS = align256(NA_L0_CNT + 4ull * NA_MAX_ROOTS);
// the two sides' exclusive scans, each with its total: nw + 1 and n - nw + 1 words
constexpr u64 NA_L1_PL = align256(NA_L0_OFFS + 8ull * (NA_MAX_ROOTS + 2));
constexpr u64 NA_L1_GRP = align256(NA_L1_PL + 3ull * NA_MAX_CHILDREN * 16);
constexpr u64 NA_L1_REM = align256(NA_L1_GRP + 4ull * NA_MAX_CHILDREN);
constexpr u64 NA_STATUS = align256(NA_L1_REM + 1ull * NA_MAX_CHILDREN);
constexpr u64 NA_STATUS_WORDS = NA_MAX_ROOTS / SCAN_TILE + 2;
constexpr u64 NA_CTRL = align256(NA_STATUS + 8 * NA_STATUS_WORDS);
// control words: [0..3] partition counters, [4..15] tickets (8 used), [16] flags
constexpr u64 NA_CTRL_WORDS = 32;
constexpr u64 NA_SCRATCH_BYTES = align256(NA_CTRL + 4 * NA_CTRL_WORDS);
static_assert(NA_SCRATCH_BYTES <= 60ull << 20, "scratch over its stated 60 MiB");

enum : u32 { NA_BAD_POSITION = 1, NA_BAD_DEPTH = 2, NA_NOT_SET_UP = 4 };
constexpr u32 NA_MAGIC = 0x9A11A10Cu;

}  // namespace

// In host code this name is only a stand-in for the device array; the device
// address comes from cudaGetSymbolAddress, on every call.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_SCRATCH_BYTES];
// NA_MAGIC once this device's move tables were uploaded.  A device reset
// reloads the module: the marker reads 0 again and the next call uploads
// the tables again instead of counting with empty ones.
static __device__ u32 g_na_ready;

namespace {

// one king per side, no overlapping piece sets, depth within 0..3; and the
// set-up marker of this device
__global__ void k_na_validate(const Pos* __restrict__ pos, const unsigned char* __restrict__ depths, u32 n,
                              u32* flags)
{
    if (blockIdx.x == 0 && threadIdx.x == 0 && g_na_ready != NA_MAGIC) atomicOr(flags, NA_NOT_SET_UP);
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Pos b = pos[i];
        const u64 pawns = b.p & INNER;
        const u64 occ = pawns | b.n | b.bq | b.rq | b.k;
        const bool ok = !(pawns & (b.n | b.bq | b.rq | b.k)) && !(b.n & (b.bq | b.rq | b.k)) &&
                        !((b.bq | b.rq) & b.k) && !(b.w & ~occ) && __popcll(b.k & b.w) == 1 &&
                        __popcll(b.k & ~b.w) == 1;
        if (!ok) atomicOr(flags, NA_BAD_POSITION);
        if (depths[i] > NA_MAX_DEPTH) atomicOr(flags, NA_BAD_DEPTH);
    }
}

struct NaDevice {
    bool ready = false;
    unsigned char* scratch = nullptr;
    int sms = 0;
};
NaDevice g_na_dev[64];
std::mutex g_na_mu;

struct NaViews {
    LevelView l0, l1;
    u32* cnt0;
    u64* offs0;
    u64* status;
    u32* ctrl;
};

NaViews views(unsigned char* s)
{
    NaViews v;
    v.l0.pl0 = (ulonglong2*)(s + NA_L0_PL);
    v.l0.pl1 = v.l0.pl0 + NA_MAX_ROOTS;
    v.l0.pl2 = v.l0.pl1 + NA_MAX_ROOTS;
    v.l0.grp = (u32*)(s + NA_L0_GRP);
    v.l0.rem = s + NA_L0_REM;
    v.l1.pl0 = (ulonglong2*)(s + NA_L1_PL);
    v.l1.pl1 = v.l1.pl0 + NA_MAX_CHILDREN;
    v.l1.pl2 = v.l1.pl1 + NA_MAX_CHILDREN;
    v.l1.grp = (u32*)(s + NA_L1_GRP);
    v.l1.rem = s + NA_L1_REM;
    v.cnt0 = (u32*)(s + NA_L0_CNT);
    v.offs0 = (u64*)(s + NA_L0_OFFS);
    v.status = (u64*)(s + NA_STATUS);
    v.ctrl = (u32*)(s + NA_CTRL);
    return v;
}

// per-device set-up, with that device current: the scratch array's device
// address (looked up on every call, so a device reset that moves the module
// is followed) and, the first time and whenever the address changed or a
// kernel found the set-up marker cleared, this translation unit's copy of the
// move tables (knight and king moves, and the magic tables the count reads the
// king's rays from) and the marker
int na_setup(int dev, bool force, NaDevice*& out)
{
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (dev < 0 || dev >= 64) {
        set_error("pg_perft_batch_noalloc: device %d out of range", dev);
        return PG_ERR_INVALID_ARGUMENT;
    }
    NaDevice& d = g_na_dev[dev];
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        set_error("cudaGetSymbolAddress(g_noalloc_scratch) failed: %s", cudaGetErrorString(e));
        return PG_ERR_CUDA;
    }
    if (!d.ready || force || p != (void*)d.scratch) {
        d.ready = false;
        const HostTables* t = host_tables();
        if (!t) {
            set_error("move table construction failed");
            return PG_ERR_CUDA;
        }
        e = upload_static_tables(*t);
        if (e != cudaSuccess) {
            set_error("move table upload failed: %s", cudaGetErrorString(e));
            return PG_ERR_CUDA;
        }
        e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) {
            set_error("device query failed: %s", cudaGetErrorString(e));
            return PG_ERR_CUDA;
        }
        const u32 magic = NA_MAGIC;
        e = cudaMemcpyToSymbol(g_na_ready, &magic, sizeof(magic));
        if (e != cudaSuccess) {
            set_error("set-up marker upload failed: %s", cudaGetErrorString(e));
            return PG_ERR_CUDA;
        }
        d.scratch = (unsigned char*)p;
        d.ready = true;
    }
    out = &d;
    return PG_OK;
}

int grid_of(const void* fn, int T, int smem, u64 items, int sms)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, T, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const u64 want = (items + T - 1) / T;
    return (int)std::max<u64>(1, std::min<u64>(want, (u64)per_sm * sms));
}

// the view of lv from node k on
LevelView from_node(const LevelView& lv, u64 k)
{
    LevelView r = lv;
    r.pl0 += k;
    r.pl1 += k;
    r.pl2 += k;
    r.grp += k;
    r.rem += k;
    return r;
}

template <int S>
void launch_leaf_na(const LevelView& lv, u32 start, u32 n, u64* out, u32* ticket, cudaStream_t st, int sms)
{
    constexpr int Q = NA_T * 32;
    using L = BlockSmem<SlKS, NA_T, Q>;
    auto fn = k_leaf<S, SlKS, NA_T, Q>;
    fn<<<grid_of((const void*)fn, NA_T, L::bytes, n, sms), NA_T, L::bytes, st>>>(lv, start, n, out, ticket, 2u);
}

template <int S>
void launch_expand_na(const LevelView& in, u32 start, u32 a, u32 b, const u64* offs, const LevelView& out,
                      u32* ticket, cudaStream_t st, int sms)
{
    constexpr int Q = NA_T * 32;
    using L = BlockSmem<SlKS, NA_T, Q>;
    auto fn = k_expand<S, SlKS, NA_T, Q>;
    fn<<<grid_of((const void*)fn, NA_T, L::bytes, b - a, sms), NA_T, L::bytes, st>>>(in, start, a, b, offs, out,
                                                                                      ticket, nullptr);
}

template <int S>
void launch_count_na(const LevelView& lv, u32 start, u32 n, u32* cnt, cudaStream_t st, int sms)
{
    auto fn = k_count_level<S, SlKS>;
    fn<<<grid_of((const void*)fn, 256, 0, n, sms), 256, 0, st>>>(lv, start, n, cnt, 3u);
}

}  // namespace
}  // namespace pg

using namespace pg;

#define NA_CUDA(call)                                                                   \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            set_error("%s failed: %s", #call, cudaGetErrorString(e_));                  \
            return PG_ERR_CUDA;                                                         \
        }                                                                               \
    } while (0)

extern "C" int pg_perft_batch_noalloc(const pg_board* d_pos, const uint8_t* d_depths, uint32_t n,
                                      uint64_t* d_out, void* stream)
{
    if (n == 0) return PG_OK;
    if (!d_pos || !d_depths || !d_out) {
        set_error("null argument");
        return PG_ERR_INVALID_ARGUMENT;
    }
    if (n > NA_MAX_ROOTS) {
        set_error("pg_perft_batch_noalloc: %u positions exceed the maximum of %u per call", n, NA_MAX_ROOTS);
        return PG_ERR_CAPACITY;
    }
    int dev = 0;
    NA_CUDA(cudaGetDevice(&dev));
    cudaStream_t st = (cudaStream_t)stream;
    const Pos* pos = (const Pos*)d_pos;
    u64* out = (u64*)d_out;
    NaDevice* d = nullptr;
    u32 head[17];
    NaViews v;
    for (int attempt = 0;; attempt++) {
        int r = na_setup(dev, attempt > 0, d);
        if (r != PG_OK) return r;
        v = views(d->scratch);
        u32* ctrl = v.ctrl;
        // everything that must start at zero: the output, the counters, the
        // scan status words (the array keeps the previous call's contents)
        NA_CUDA(cudaMemsetAsync(out, 0, (size_t)n * sizeof(u64), st));
        NA_CUDA(cudaMemsetAsync(ctrl, 0, NA_CTRL_WORDS * 4, st));
        NA_CUDA(cudaMemsetAsync(ctrl + 2, 0xFF, 4, st));  // min depth starts at UINT_MAX
        const int g = (int)std::min<u32>((n + 255) / 256, 1024);
        k_na_validate<<<g, 256, 0, st>>>(pos, d_depths, n, ctrl + 16);
        k_partition_roots<<<g, 256, 0, st>>>(pos, d_depths, n, v.l0, ctrl);
        NA_CUDA(cudaGetLastError());
        NA_CUDA(cudaMemcpyAsync(head, ctrl, sizeof(head), cudaMemcpyDeviceToHost, st));
        NA_CUDA(cudaStreamSynchronize(st));
        if (!(head[16] & NA_NOT_SET_UP)) break;
        if (attempt > 0) {
            set_error("pg_perft_batch_noalloc: device set-up did not take effect");
            return PG_ERR_CUDA;
        }
    }
    if (head[16] & NA_BAD_POSITION) {
        set_error("pg_perft_batch_noalloc: a position is not a valid board");
        return PG_ERR_INVALID_POSITION;
    }
    if (head[16] & NA_BAD_DEPTH) {
        set_error("pg_perft_batch_noalloc: depths are limited to 0..%d", NA_MAX_DEPTH);
        return PG_ERR_CAPACITY;
    }
    const u32 nw = head[0], maxd = head[3];
    u32* ctrl = v.ctrl;
    u32* tickets = ctrl + 4;
    // depth-3 positions: count and scan both sides' children first, so that
    // the children limit is checked before any leaf kernel runs
    u64 total[2] = {0, 0};
    u64* offs[2] = {v.offs0, v.offs0 + nw + 1};
    if (maxd == 3) {
        for (int side = 0; side < 2; side++) {
            const u32 start = side ? nw : 0, cnt = side ? n - nw : nw;
            if (!cnt) continue;
            if (side) launch_count_na<1>(v.l0, start, cnt, v.cnt0, st, d->sms);
            else launch_count_na<0>(v.l0, start, cnt, v.cnt0, st, d->sms);
            NA_CUDA(cudaMemsetAsync(v.status, 0, NA_STATUS_WORDS * 8, st));
            const u32 tiles = (cnt + SCAN_TILE - 1) / SCAN_TILE;
            k_scan<<<tiles, SCAN_T, 0, st>>>(v.cnt0, cnt, offs[side], v.status, tickets + side, ctrl + 16);
            NA_CUDA(cudaGetLastError());
            NA_CUDA(cudaMemcpyAsync(&total[side], offs[side] + cnt, sizeof(u64), cudaMemcpyDeviceToHost, st));
        }
        u32 flags = 0;
        NA_CUDA(cudaMemcpyAsync(&flags, ctrl + 16, sizeof(flags), cudaMemcpyDeviceToHost, st));
        NA_CUDA(cudaStreamSynchronize(st));
        if (flags) {
            set_error("pg_perft_batch_noalloc: device error flags 0x%x", flags);
            return PG_ERR_DEVICE_TIMEOUT;
        }
        if (total[0] + total[1] > NA_MAX_CHILDREN) {
            set_error("pg_perft_batch_noalloc: the depth-3 positions have %llu children, over the maximum of %u "
                      "per call",
                      (unsigned long long)(total[0] + total[1]), NA_MAX_CHILDREN);
            return PG_ERR_CAPACITY;
        }
    }
    // level 0: nodes with remaining depth <= 2 finish in the leaf kernel
    launch_leaf_na<0>(v.l0, 0, nw, out, tickets + 2, st, d->sms);
    launch_leaf_na<1>(v.l0, nw, n - nw, out, tickets + 3, st, d->sms);
    NA_CUDA(cudaGetLastError());
    if (maxd == 3) {
        // white-to-move positions' children at [0, total0), black's after them
        const LevelView l1b = from_node(v.l1, total[0]);
        if (total[0]) {
            launch_expand_na<0>(v.l0, 0, 0, nw, offs[0], v.l1, tickets + 4, st, d->sms);
            launch_leaf_na<1>(v.l1, 0, (u32)total[0], out, tickets + 5, st, d->sms);
        }
        if (total[1]) {
            launch_expand_na<1>(v.l0, nw, 0, n - nw, offs[1], l1b, tickets + 6, st, d->sms);
            launch_leaf_na<0>(l1b, 0, (u32)total[1], out, tickets + 7, st, d->sms);
        }
        NA_CUDA(cudaGetLastError());
    }
    NA_CUDA(cudaStreamSynchronize(st));
    return PG_OK;
}
