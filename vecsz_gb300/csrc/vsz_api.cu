// C ABI of the library (include/vecsz_gb300.h): argument checks, workspace layout and the
// stream-ordered compress / decompress pipelines built from the kernels in dq_*.cu and huffman.cu.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "api_common.cuh"
#include "host_tree.h"
#include "vsz_device.cuh"
#include "vsz_huffman.h"
#include "vsz_kernels.h"
#include "vsz_profile.h"

using namespace vsz;
using namespace vsz::api;

static_assert(sizeof(Consts) <= VSZ_CONSTS_BYTES, "Consts must fit VSZ_CONSTS_BYTES");

namespace vsz {
// A tree builder for the calling thread's next compress calls (VSZ_TREE_HOST / _DEVICE), or -1
// for the process setting: the host-buffer operations take the device builder (vsz_host.cu).
thread_local int t_tree_builder = -1;
void set_thread_tree_builder(int which) { t_tree_builder = which; }
int g_sms[64];
int num_sms() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!g_sms[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        g_sms[dev] = v > 0 ? v : 152;
    }
    return g_sms[dev];
}
}  // namespace vsz

namespace {

__global__ void k_finalize(FinalizeArgs f) { finalize_field(f, blockIdx.x, gridDim.x); }

__global__ void k_check_zeros(const unsigned long long* total_zeros, unsigned long long n_out, int* status) {
    if (*total_zeros != n_out) set_status(status, VSZ_ERR_CORRUPT);
}

__global__ void k_copy_status(const int* from, const Consts* c, int* to) {
    int st = c->status != VSZ_OK ? c->status : *from;
    *to    = st;
}

// ---- workspace layouts ------------------------------------------------------------------------

struct CompressWs {
    Consts* consts;
    uint32_t* mm;
    int* status;
    unsigned long long* hist;
    uint16_t* code;
    uint8_t* seg_count;
    float* scratch;
    unsigned long long* g_tile_status;
    uint32_t* g_counter;
    uint32_t* g_seg_off;              // split outlier copy: offset of each segment within its tile
    unsigned long long* g_tile_base;  // and each tile's first outlier
    unsigned long long* n_out;
    uint8_t* build_scratch;
    uint8_t* cb_block;
    unsigned long long* cb_word;
    uint8_t* cb_len;
    uint32_t* build_info;
    unsigned long long* e_chunk_off;
    unsigned long long* e_scan_status;
    unsigned long long* e_edge_idx;
    uint32_t* e_edge_bits;
    uint32_t* e_counter;
    unsigned long long* total_bits;
    uint16_t* chunk_bits;
    size_t n_chunks;
    uint8_t* pad_ws;   // padding: reduction state of the global value
    float* halo_g;     // padding, global mode: the value the blocks predict from
    size_t bytes;
};

// dict: histogram / codebook symbols (symbol_count)
CompressWs layout_compress(const Geometry& g, int dict, uint8_t* base, size_t cap) {
    Bump b{base, cap};
    CompressWs w{};
    w.consts    = b.take<Consts>(1);
    w.mm        = b.take<uint32_t>(4);
    w.status    = b.take<int>(4);
    w.hist      = b.take<unsigned long long>(dict);
    w.code      = b.take<uint16_t>(g.n + 8);
    w.seg_count = b.take<uint8_t>(g.nseg + 16);
    w.scratch   = b.take<float>(g.nseg * kSegX);
    size_t gt   = (g.nseg + 4095) / 4096 + 1;
    w.g_tile_status = b.take<unsigned long long>(gt);
    w.g_counter = b.take<uint32_t>(4);
    w.g_seg_off = b.take<uint32_t>(g.nseg + 16);
    w.g_tile_base = b.take<unsigned long long>(gt);
    w.n_out     = b.take<unsigned long long>(1);
    w.build_scratch = b.take<uint8_t>(huff_build_scratch_bytes(dict));
    // codebook block [cb_word dict x u64][info 4 x u32][cb_len dict x u8]: one copy from the host
    // tree builder's staging fills it
    uint8_t* cb  = b.take<uint8_t>(codebook_block_bytes(dict));
    w.cb_block   = cb;
    w.cb_word    = reinterpret_cast<unsigned long long*>(cb);
    w.build_info = cb ? reinterpret_cast<uint32_t*>(cb + 8 * (size_t)dict) : nullptr;
    w.cb_len     = cb ? cb + 8 * (size_t)dict + 16 : nullptr;
    w.n_chunks   = (g.n + kChunkSyms - 1) / kChunkSyms;
    w.e_chunk_off   = b.take<unsigned long long>(w.n_chunks + 1);
    w.e_scan_status = b.take<unsigned long long>(scan_tmp_tiles(w.n_chunks) + 1);
    w.e_edge_idx  = b.take<unsigned long long>(2 * w.n_chunks + 2);
    w.e_edge_bits = b.take<uint32_t>(2 * w.n_chunks + 2);
    w.e_counter  = b.take<uint32_t>(4);
    w.total_bits = b.take<unsigned long long>(1);
    w.chunk_bits = b.take<uint16_t>(w.n_chunks + 8);
    w.pad_ws     = b.take<uint8_t>(pad_ws_bytes());
    w.halo_g     = b.take<float>(4);
    w.bytes      = b.off + 256;
    return w;
}


struct DecompressWs {
    Consts* consts;
    uint32_t* mm;
    int* status;
    uint32_t* table;
    uint32_t* table2;
    uint32_t* child;
    uint32_t* node_sym;
    uint32_t* parent;
    uint32_t* walk;
    uint32_t* tinfo;
    uint16_t* code;
    uint32_t* seg_zero;
    unsigned long long* seg_off;
    uint32_t* chunk_zero;
    unsigned long long* chunk_off;
    unsigned long long* scan_status;
    uint32_t* scan_counter;
    unsigned long long* scan_total;
    unsigned long long* chunk_start;  // index path
    unsigned long long* s_start;      // sync path
    unsigned long long* s_exit_a;
    unsigned long long* s_exit_b;
    uint32_t* s_count;
    unsigned long long* s_out_begin;
    int* s_changed;
    float* outliers;
    uint32_t* blk_zero;             // zero codes per (row, x-block of 8): small 3D fields only
    unsigned long long* blk_off;    // their exclusive scan (outlier rank of each row's block)
    uint32_t* redo;  // units of the separable reverse Lorenzo that the reference-order kernel redoes
    unsigned long long* dq_cache;  // the last dequantization check (k_dq_mul_verify), at a fixed offset
    size_t bytes;
};

DecompressWs layout_decompress(const Geometry& g, int dict, size_t payload_bytes, size_t n_out, size_t n_index_chunks,
                               uint8_t* base, size_t cap) {
    Bump b{base, cap};
    DecompressWs w{};
    uint32_t maxn = (uint32_t)(2 * dict);
    w.consts   = b.take<Consts>(1);
    w.dq_cache = b.take<unsigned long long>(4);  // offset 256 whatever the field: kept across calls
    w.mm       = b.take<uint32_t>(4);
    w.status   = b.take<int>(4);
    w.table    = b.take<uint32_t>(1u << kDecBits);
    w.table2   = b.take<uint32_t>(table2_capacity(maxn));
    w.child    = b.take<uint32_t>(2 * (size_t)maxn);
    w.node_sym = b.take<uint32_t>(maxn);
    w.parent   = b.take<uint32_t>(maxn);
    w.walk     = b.take<uint32_t>(maxn);
    w.tinfo    = b.take<uint32_t>(4);
    w.code     = b.take<uint16_t>(g.n + 8);
    uint32_t nxs = (g.d0 + 255) / 256;
    size_t nsegd = g.nrows * nxs;
    w.seg_zero = b.take<uint32_t>(nsegd + 1);
    w.seg_off  = b.take<unsigned long long>(nsegd + 1);
    w.chunk_zero = b.take<uint32_t>(n_index_chunks + 1);
    w.chunk_off  = b.take<unsigned long long>(n_index_chunks + 1);
    const size_t nblk = (g.ndim == 3 && g.n <= kW8MaxN) ? g.nrows * ((g.d0 + 7) / 8) : 0;
    w.blk_zero = b.take<uint32_t>(nblk + 1);
    w.blk_off  = b.take<unsigned long long>(nblk + 1);
    size_t nsync = (payload_bytes * 8 + kSyncBits - 1) / kSyncBits + 1;
    size_t scan_n = nsegd > nblk ? nsegd : nblk;
    if (n_index_chunks > scan_n) scan_n = n_index_chunks;
    if (nsync > scan_n) scan_n = nsync;
    w.scan_status  = b.take<unsigned long long>(scan_tmp_tiles(scan_n) + 1);
    w.scan_counter = b.take<uint32_t>(4);
    w.scan_total   = b.take<unsigned long long>(1);
    w.chunk_start  = b.take<unsigned long long>(n_index_chunks + 1);
    w.s_start      = b.take<unsigned long long>(nsync);
    w.s_exit_a     = b.take<unsigned long long>(nsync);
    w.s_exit_b     = b.take<unsigned long long>(nsync);
    w.s_count      = b.take<uint32_t>(nsync);
    w.s_out_begin  = b.take<unsigned long long>(nsync);
    w.s_changed    = b.take<int>(4);
    w.outliers     = b.take<float>(n_out + 4);
    {
        const size_t units8 = (size_t)nxs * ((g.d1 + 7) / 8) * ((g.d2 + 7) / 8);  // block-8 warp units
        w.redo = b.take<uint32_t>(units8 + 2);
    }
    w.bytes        = b.off + 256;
    return w;
}

// Decode n codes from a Huffman section at d_huff.  Index path when chunk_bits != null.
int decode_codes(const uint8_t* d_huff, size_t huff_bytes, uint32_t node_count, size_t tree_bytes, size_t n, int dict,
                 const uint16_t* chunk_bits, size_t n_index_chunks, uint32_t chunk_syms, const DecompressWs& w,
                 uint32_t* seg_zero, uint32_t d0, cudaStream_t st) {
    const uint8_t* payload   = d_huff + 8 + tree_bytes;
    size_t payload_bytes     = huff_bytes - 8 - tree_bytes;
    unsigned long long pbits = (unsigned long long)payload_bytes * 8ull;
    uint32_t nxs             = (d0 + 255) / 256;
    HuffTableArgs ta{};
    ta.huff = d_huff;
    ta.huff_bytes = huff_bytes;
    ta.dict = dict;
    ta.max_nodes = (uint32_t)(2 * dict - 1);
    ta.table = w.table;
    ta.child = w.child;
    ta.node_sym = w.node_sym;
    ta.parent = w.parent;
    ta.walk = w.walk;
    ta.table2 = w.table2;
    ta.info = w.tinfo;
    ta.status = w.status;
    {
        StageTimer t(kStDecTable, st);
        VSZ_TRY(launch_huff_table(ta, st));
    }
    if (node_count == 1) {
        // one-symbol tree: constant output (src/huffman.hh:348-352)
        return launch_huff_const(w.code, n, w.tinfo, seg_zero, d0, nxs, w.status, st, num_sms());
    }
    HuffDecodeArgs da{};
    da.payload = payload;
    da.payload_bits = pbits;
    da.table = w.table;
    da.table2 = w.table2;
    da.child = w.child;
    da.node_sym = w.node_sym;
    da.codes = w.code;
    da.n = n;
    da.seg_zero = seg_zero;
    da.d0 = d0;
    da.nxs = nxs;
    da.max_nodes = (uint32_t)(2 * dict - 1);
    da.walk = w.walk;
    da.nodes = node_count;
    da.walk_smem = (dict <= 16384 && node_count < 32768u) ? 1 : 0;
    // the window decoder takes trees whose codewords are at most 32 bits; VSZ_DECODE_NO_WINDOW
    // sends every tree to the general indexed decoder (tests of that path)
    da.tree_info = getenv("VSZ_DECODE_NO_WINDOW") ? nullptr : w.tinfo;
    da.status = w.status;
    if (chunk_bits) {
        {
            StageTimer t(kStDecScanIndex, st);
            VSZ_TRY(launch_scan_u16(chunk_bits, w.chunk_start, n_index_chunks, w.scan_status, w.scan_counter, nullptr,
                                    w.status, st));
        }
        da.start_bit = w.chunk_start;
        da.chunk_len = chunk_bits;
        da.chunk_zero = w.chunk_zero;
        da.out_begin = nullptr;
        da.nsym = nullptr;
        da.nchunks = n_index_chunks;
        da.chunk_syms = chunk_syms;
        StageTimer t(kStHuffDecode, st);
        return launch_huff_decode(da, st);
    }
    // self-synchronising path
    HuffSyncArgs sa{};
    sa.payload = payload;
    sa.payload_bits = pbits;
    sa.table = w.table;
    sa.table2 = w.table2;
    sa.child = w.child;
    sa.node_sym = w.node_sym;
    sa.nchunks = (size_t)((pbits + kSyncBits - 1) / kSyncBits);
    sa.chunk_bits = kSyncBits;
    sa.start = w.s_start;
    sa.exit_a = w.s_exit_a;
    sa.count = w.s_count;
    sa.max_nodes = (uint32_t)(2 * dict - 1);
    sa.status = w.status;
    if (sa.nchunks == 0) return VSZ_ERR_CORRUPT;
    VSZ_TRY(launch_huff_sync_init(sa, st));
    unsigned long long* ein  = w.s_exit_a;
    unsigned long long* eout = w.s_exit_b;
    for (size_t round = 0; round < sa.nchunks + 2; round++) {
        VSZ_CUDA(cudaMemsetAsync(w.s_changed, 0, sizeof(int), st));
        VSZ_TRY(launch_huff_sync_round(sa, ein, eout, w.s_changed, st));
        int changed = 0;
        VSZ_CUDA(cudaMemcpyAsync(&changed, w.s_changed, sizeof(int), cudaMemcpyDeviceToHost, st));
        VSZ_CUDA(cudaStreamSynchronize(st));
        unsigned long long* t = ein;
        ein  = eout;
        eout = t;
        if (!changed) break;
    }
    VSZ_TRY(launch_scan_u32(w.s_count, w.s_out_begin, sa.nchunks, w.scan_status, w.scan_counter, w.scan_total,
                            w.status, st));
    unsigned long long total = 0;
    VSZ_CUDA(cudaMemcpyAsync(&total, w.scan_total, 8, cudaMemcpyDeviceToHost, st));
    VSZ_CUDA(cudaStreamSynchronize(st));
    if (total < n) return VSZ_ERR_CORRUPT;
    da.start_bit = w.s_start;
    da.out_begin = w.s_out_begin;
    da.nsym = w.s_count;
    da.nchunks = sa.nchunks;
    da.chunk_syms = 0;
    return launch_huff_decode(da, st);
}

// ---- Huffman tree on the host, stream-ordered ---------------------------------------------------
// The tree build replays the reference's binary heap one operation at a time: ~20k dependent,
// branchy steps on a few KB for a 1024-symbol dictionary.  One GPU thread runs that chain at
// shared-memory latency; a host core runs it from L1, several times faster.  The step stays in
// stream order as one kernel, k_tree_handoff: it writes the histogram into mapped pinned staging,
// posts a request number there and waits (bounded) for the host worker thread, which polls the
// staging areas of queued requests, builds the tree and answers with the same number; the kernel
// then copies the codebook into the workspace and the serialised tree into the archive.  Nothing
// returns to the caller's thread and nothing synchronises.  Under stream capture (a CUDA graph)
// the device builder k_huff_build is used.
//
// A stream host function (cudaLaunchHostFunc) between two copy kernels did the same at 0.12 ms a
// build; the handoff takes 0.056 ms.  The small transfers are loads and stores of a kernel to the
// mapped area, not copy-engine copies: a copy engine serves its queue in order, so with several
// streams in flight a few-KB histogram or codebook copy would wait behind another stream's
// field-sized transfer, and the Huffman stage of this compress with it.

std::atomic<int> g_tree_builder{-1};

int tree_builder() {
    if (t_tree_builder >= 0) return t_tree_builder;
    int v = g_tree_builder.load(std::memory_order_relaxed);
    if (v < 0) {
        v               = VSZ_TREE_HOST;
        const char* env = getenv("VSZ_TREE_BUILD");
        if (env && !strcmp(env, "device")) v = VSZ_TREE_DEVICE;
        g_tree_builder.store(v, std::memory_order_relaxed);
    }
    return v;
}

// One pinned staging area: [hist dict x u64][codebook block][tree head][flags: request, answer].
// The stream hands the histogram to the host and takes the codebook and tree back in one kernel
// (k_tree_handoff): it posts the histogram and a request number in the staging area and waits,
// bounded, for a host worker thread to answer with the same number.  A slot is reused once the
// event recorded after its kernel has completed and the worker has let it go.
struct TreeSlot {
    int device    = -1;
    int dict_cap  = 0;
    int dict      = 0;
    int hdr_dict  = 0;
    bool reserved = false;
    uint8_t* pinned = nullptr;
    uint8_t* pinned_dev = nullptr;  // the same area as the device addresses it
    cudaEvent_t done = nullptr;
    size_t hist_off = 0, cb_off = 0, head_off = 0, flags_off = 0;
    uint32_t seq = 0;                    // this use's request number (never 0)
    bool dead    = false;                // its event failed (e.g. the device was reset): never reused
    std::atomic<bool> in_worker{false};  // queued to the worker, not yet answered or dropped
    std::atomic<bool> cancel{false};     // the enqueue failed: the worker drops the request
};

// Copies the histogram (hist_bytes) into the staging area, posts `seq` in flags[0], waits until the
// host answers `seq` in flags[1] (or wait_ns pass: VSZ_ERR_TIMEOUT, nothing copied back), then
// copies the codebook block and the tree head to the device.  One block of kHandoffThreads: every
// thread issues all its reads of host memory before it stores anything, in 16-byte pieces, so
// the answer crosses the host link in about one round trip even when bulk copies of other
// streams queue ahead of it.
constexpr int kHandoffThreads = 1024;
constexpr int kHandoffUnroll  = 4;

__global__ void __launch_bounds__(kHandoffThreads)
    k_tree_handoff(const uint8_t* __restrict__ hist, uint8_t* pin, size_t hist_off, size_t hist_bytes, size_t cb_off,
                   uint8_t* __restrict__ cb_block, size_t cb_bytes, size_t head_off, uint8_t* __restrict__ huff_out,
                   size_t head_bytes, size_t flags_off, uint32_t seq, long long wait_ns, int* status) {
    __shared__ int s_ok;
    const unsigned t = threadIdx.x;
    // 8-byte histogram words into the 256-byte aligned staging block (bytes from a workspace that
    // the caller did not align)
    if ((reinterpret_cast<uintptr_t>(hist) & 7u) == 0) {
        for (size_t i = t; i < hist_bytes / 8; i += blockDim.x)
            reinterpret_cast<unsigned long long*>(pin + hist_off)[i] = reinterpret_cast<const unsigned long long*>(hist)[i];
    } else {
        for (size_t i = t; i < hist_bytes; i += blockDim.x) pin[hist_off + i] = hist[i];
    }
    __threadfence_system();
    __syncthreads();
    volatile uint32_t* flags = reinterpret_cast<volatile uint32_t*>(pin + flags_off);
    if (t == 0) {
        flags[0] = seq;
        __threadfence_system();
        unsigned long long t0, now;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
        bool ok = false;
        for (;;) {
            if (flags[1] == seq) {
                ok = true;
                break;
            }
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
            if ((long long)(now - t0) > wait_ns) break;
            __nanosleep(500);
        }
        __threadfence_system();
        if (!ok) set_status(status, VSZ_ERR_TIMEOUT);
        s_ok = ok;
    }
    __syncthreads();
    if (!s_ok) return;
    // the answer, read past the caches (the host wrote it after the kernel started): the codebook
    // block (16-byte aligned at both ends but its tail) and the head (aligned in the staging area,
    // not in the archive: stored byte by byte)
    const bool cb16       = (reinterpret_cast<uintptr_t>(cb_block) & 15u) == 0;
    const uint4* cb_src   = reinterpret_cast<const uint4*>(pin + cb_off);
    const uint4* head_src = reinterpret_cast<const uint4*>(pin + head_off);
    const size_t n_cb = cb_bytes / 16, n_head = (head_bytes + 15) / 16, n_all = n_cb + n_head;
    for (size_t base = 0; base < n_all; base += (size_t)kHandoffUnroll * blockDim.x) {
        uint4 v[kHandoffUnroll];
#pragma unroll
        for (int u = 0; u < kHandoffUnroll; u++) {
            const size_t i = base + (size_t)u * blockDim.x + t;
            if (i < n_all) v[u] = __ldcv(i < n_cb ? cb_src + i : head_src + (i - n_cb));
        }
#pragma unroll
        for (int u = 0; u < kHandoffUnroll; u++) {
            const size_t i = base + (size_t)u * blockDim.x + t;
            const uint32_t w[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
            if (i < n_cb && cb16) {
                reinterpret_cast<uint4*>(cb_block)[i] = v[u];
            } else if (i < n_cb) {
#pragma unroll
                for (int k = 0; k < 16; k++) cb_block[i * 16 + k] = (uint8_t)(w[k >> 2] >> (8 * (k & 3)));
            } else if (i < n_all) {
                const size_t o = (i - n_cb) * 16;
#pragma unroll
                for (int k = 0; k < 16; k++)
                    if (o + k < head_bytes) huff_out[o + k] = (uint8_t)(w[k >> 2] >> (8 * (k & 3)));
            }
        }
    }
    for (size_t i = n_cb * 16 + t; i < cb_bytes; i += blockDim.x)
        cb_block[i] = __ldcv(reinterpret_cast<const unsigned char*>(pin + cb_off) + i);
}

std::mutex g_slot_mu;
std::vector<TreeSlot*> g_slots;
std::atomic<long long> g_tree_wait_ns{2000000000ll};  // the handoff's bound: 2 s

// The host side of the handoff: one thread for the process, started on first use and never
// destroyed (it may outlive static destructors).  While requests are queued it polls their
// request words and builds each tree as soon as its stream has posted the histogram.
struct TreeWorker {
    std::mutex mu;
    std::condition_variable cv;
    std::vector<TreeSlot*> queued;
    std::atomic<int> hold{0};  // test hook: leave requests unanswered while set
};

void answer_tree(TreeSlot* s) {
    const int dict = s->dict;
    uint8_t* cb    = s->pinned + s->cb_off;
    host_huffman_build(reinterpret_cast<const uint64_t*>(s->pinned + s->hist_off), dict,
                       reinterpret_cast<uint64_t*>(cb), cb + 8 * (size_t)dict + 16,
                       reinterpret_cast<uint32_t*>(cb + 8 * (size_t)dict), s->pinned + s->head_off, s->hdr_dict);
    __atomic_store_n(reinterpret_cast<uint32_t*>(s->pinned + s->flags_off) + 1, s->seq, __ATOMIC_RELEASE);
}

void tree_worker_loop(TreeWorker* w) {
    using clk = std::chrono::steady_clock;
    std::vector<std::pair<TreeSlot*, clk::time_point>> mine;
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(w->mu);
            if (mine.empty()) w->cv.wait(lk, [&] { return !w->queued.empty(); });
            for (TreeSlot* s : w->queued) mine.emplace_back(s, clk::now());
            w->queued.clear();
        }
        bool progress = false;
        for (size_t i = 0; i < mine.size();) {
            TreeSlot* s    = mine[i].first;
            bool drop      = s->cancel.load(std::memory_order_acquire);
            const uint32_t req = __atomic_load_n(reinterpret_cast<uint32_t*>(s->pinned + s->flags_off), __ATOMIC_ACQUIRE);
            if (!drop && req == s->seq && !w->hold.load(std::memory_order_relaxed)) {
                answer_tree(s);
                drop = true;
            } else if (!drop && clk::now() - mine[i].second > std::chrono::seconds(1)) {
                // not posted after a second: keep waiting unless the stream failed for good (the
                // event was recorded at enqueue; a kernel that ran would have posted first)
                cudaSetDevice(s->device);
                const cudaError_t e = cudaEventQuery(s->done);
                if (e != cudaErrorNotReady && e != cudaSuccess) {
                    cudaGetLastError();
                    drop = true;
                }
                mine[i].second = clk::now();
            }
            if (drop) {
                s->in_worker.store(false, std::memory_order_release);
                mine[i] = mine.back();
                mine.pop_back();
                progress = true;
            } else {
                i++;
            }
        }
        if (!progress) std::this_thread::yield();
    }
}

TreeWorker* tree_worker() {
    static TreeWorker* w = [] {
        TreeWorker* t = new TreeWorker();
        std::thread(tree_worker_loop, t).detach();
        return t;
    }();
    return w;
}

// Slots are made up to kTreeSlotBatch at a time from one pinned allocation (at most
// kTreeSlotBatchBytes, at least 2 slots), so that a burst of concurrent compresses (a request
// server's slots) does not pin host memory on its critical path: the first compress of a
// dictionary size makes them.  A 1024-symbol slot takes ~37 KB, a 65536-symbol one ~2.6 MB.
constexpr int kTreeSlotBatch         = 16;
constexpr size_t kTreeSlotBatchBytes = size_t(8) << 20;

TreeSlot* acquire_tree_slot(int dict) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> g(g_slot_mu);
    for (TreeSlot* s : g_slots) {
        if (s->dead || s->reserved || s->device != dev || s->dict_cap < dict) continue;
        if (s->in_worker.load(std::memory_order_acquire)) continue;  // the worker still holds it
        const cudaError_t e = cudaEventQuery(s->done);
        if (e == cudaErrorNotReady) continue;  // its kernel is still queued
        if (e != cudaSuccess) {                 // a context torn down under it: retire the slot
            cudaGetLastError();                 // and leave no error behind for the caller
            s->dead = true;
            continue;
        }
        s->reserved = true;
        return s;
    }
    const size_t cb_off    = (8 * (size_t)dict + 255) & ~(size_t)255;
    const size_t head_off  = (cb_off + codebook_block_bytes(dict) + 255) & ~(size_t)255;
    const size_t flags_off = (head_off + tree_head_max(dict) + 255) & ~(size_t)255;
    const size_t stride    = (flags_off + 64 + 255) & ~(size_t)255;
    const int batch = (int)std::max<size_t>(2, std::min<size_t>(kTreeSlotBatch, kTreeSlotBatchBytes / stride));
    uint8_t *pinned = nullptr, *pinned_dev = nullptr;
    if (cudaHostAlloc(reinterpret_cast<void**>(&pinned), stride * batch, cudaHostAllocDefault) != cudaSuccess)
        return nullptr;
    if (cudaHostGetDevicePointer(reinterpret_cast<void**>(&pinned_dev), pinned, 0) != cudaSuccess) {
        cudaGetLastError();
        cudaFreeHost(pinned);
        return nullptr;
    }
    TreeSlot* first = nullptr;
    for (int k = 0; k < batch; k++) {
        TreeSlot* s   = new TreeSlot();
        s->device     = dev;
        s->dict_cap   = dict;
        s->pinned     = pinned + k * stride;
        s->pinned_dev = pinned_dev + k * stride;
        s->hist_off   = 0;
        s->cb_off     = cb_off;
        s->head_off   = head_off;
        s->flags_off  = flags_off;
        memset(s->pinned + s->flags_off, 0, 64);
        if (cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            delete s;  // the slots made so far stay usable; the pinned block stays allocated
            break;
        }
        g_slots.push_back(s);
        if (!first) first = s;
    }
    if (first) first->reserved = true;
    return first;
}

void release_tree_slot(TreeSlot* s) {
    std::lock_guard<std::mutex> g(g_slot_mu);
    s->reserved = false;
}

// Enqueue the host build: hist (device) -> codebook block (device workspace) and
// [BE nc][BE hdr_dict][tree] at huff_out (device archive; up to tree_head_max(dict) bytes are
// written, the bytes past the tree are overwritten by the encoder that follows).
int enqueue_host_tree(const unsigned long long* hist, int dict, int hdr_dict, uint8_t* cb_block, uint8_t* huff_out,
                      int* status, cudaStream_t st) {
    TreeWorker* w = tree_worker();
    TreeSlot* s   = acquire_tree_slot(dict);
    if (!s) return VSZ_ERR_CUDA;
    s->dict     = dict;
    s->hdr_dict = hdr_dict;
    if (++s->seq == 0) s->seq = 1;
    s->cancel.store(false, std::memory_order_relaxed);
    s->in_worker.store(true, std::memory_order_release);
    {
        std::lock_guard<std::mutex> g(w->mu);
        w->queued.push_back(s);
    }
    w->cv.notify_one();
    int rc = VSZ_OK;
    k_tree_handoff<<<1, kHandoffThreads, 0, st>>>(reinterpret_cast<const uint8_t*>(hist), s->pinned_dev, s->hist_off,
                                      8 * (size_t)dict, s->cb_off, cb_block, codebook_block_bytes(dict), s->head_off,
                                      huff_out, tree_head_max(dict), s->flags_off, s->seq,
                                      g_tree_wait_ns.load(std::memory_order_relaxed), status);
    count_launch();
    if (cudaGetLastError() != cudaSuccess) {
        s->cancel.store(true, std::memory_order_release);
        rc = VSZ_ERR_CUDA;
    }
    // recorded even after a failed launch, so the slot is not reused while anything queued reads it
    if (cudaEventRecord(s->done, st) != cudaSuccess) rc = VSZ_ERR_CUDA;
    release_tree_slot(s);
    return rc;
}

bool stream_capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) return true;
    return cs != cudaStreamCaptureStatusNone;
}

}  // namespace

// =================================================================================================
extern "C" {

const char* vsz_status_string(vsz_status s) {
    switch (s) {
        case VSZ_OK: return "ok";
        case VSZ_ERR_INVALID: return "invalid argument";
        case VSZ_ERR_CUDA: return "CUDA runtime error";
        case VSZ_ERR_CORRUPT: return "corrupt archive or bitstream";
        case VSZ_ERR_CAPACITY: return "buffer or workspace too small";
        case VSZ_ERR_TIMEOUT: return "device-side wait timed out";
        case VSZ_ERR_UNSUPPORTED: return "unsupported setting";
        case VSZ_ERR_RANGE: return "zero value range (r2r)";
        case VSZ_ERR_NOMEM: return "out of memory";
        case VSZ_ERR_NO_DEVICE: return "no CUDA device";
        case VSZ_ERR_CANCELLED: return "request cancelled";
        default: return "unknown status";
    }
}

const char* vsz_version(void) { return "vecsz_gb300 0.1 (sm_103a)"; }

// The -p string, as src/argument_parser/argparse.cc:399-415 reads it: substrings select the mode
// and the value type, the first match of [0-9]*[.][0-9]+|[0-9]+ is the constant (so a sign is not
// part of it); then one mode is kept (argparse.cc:156-170).
vsz_status vsz_parse_padding(const char* spec, vsz_params* p) {
    if (!spec || !p) return VSZ_ERR_INVALID;
    const std::string t(spec);
    const bool global = t.find("global") != std::string::npos;
    const bool block  = t.find("block") != std::string::npos;
    const bool edge   = t.find("edge") != std::string::npos;
    int type          = VSZ_PADV_CONST;
    if (t.find("max") != std::string::npos) type = VSZ_PADV_MAX;
    if (t.find("min") != std::string::npos) type = VSZ_PADV_MIN;
    if (t.find("avg") != std::string::npos) type = VSZ_PADV_AVG;
    if (t.find("constant") != std::string::npos) type = VSZ_PADV_CONST;
    float cst = 0.0f;
    auto digit = [&](size_t i) { return i < t.size() && t[i] >= '0' && t[i] <= '9'; };
    for (size_t i = 0; i < t.size(); i++) {
        size_t j = i;
        while (digit(j)) j++;
        size_t end = 0;
        if (j < t.size() && t[j] == '.' && digit(j + 1)) {  // [0-9]*[.][0-9]+
            end = j + 1;
            while (digit(end)) end++;
        } else if (j > i) {  // [0-9]+
            end = j;
        }
        if (end) {
            cst = strtof(t.substr(i, end - i).c_str(), nullptr);
            break;
        }
    }
    p->pad_mode     = global ? VSZ_PAD_GLOBAL : (block ? VSZ_PAD_BLOCK : (edge ? VSZ_PAD_EDGE : VSZ_PAD_NONE));
    p->pad_type     = type;
    p->pad_constant = cst;
    return VSZ_OK;
}

size_t vsz_pad_count(int ndim, const size_t dims[3], int block_size, int pad_mode) {
    if (!valid_dims(ndim, dims) || block_size <= 0) return 0;
    Geometry g = make_geometry(ndim, dims);
    const uint32_t d3[3] = {g.d0, g.d1, g.d2};
    return pad_count(ndim, d3, block_size, pad_mode);
}

vsz_status vsz_eb_setup(const vsz_params* p, const float* d_in, size_t n, void* d_consts, void* d_tmp, void* stream) {
    if (!p || !d_consts || !d_tmp) return VSZ_ERR_INVALID;
    if (p->mode == VSZ_MODE_R2R && (!d_in || n == 0)) return VSZ_ERR_INVALID;
    if (!(p->eb > 0.0)) return VSZ_ERR_INVALID;
    return launch_eb_setup(p->mode, p->eb, d_in, n, reinterpret_cast<Consts*>(d_consts),
                           reinterpret_cast<uint32_t*>(d_tmp), S(stream));
}

vsz_status vsz_consts_read(const void* d_consts, double h_out[4], int* h_status, void* stream) {
    Consts c;
    VSZ_CUDA(cudaMemcpyAsync(&c, d_consts, sizeof(Consts), cudaMemcpyDeviceToHost, S(stream)));
    VSZ_CUDA(cudaStreamSynchronize(S(stream)));
    if (h_out) {
        h_out[0] = c.eb_final;
        h_out[1] = c.c_d;
        h_out[2] = c.r_d;
        h_out[3] = c.range;
    }
    if (h_status) *h_status = c.status;
    return VSZ_OK;
}

size_t vsz_outlier_segments(int ndim, const size_t dims[3]) {
    if (!valid_dims(ndim, dims)) return 0;
    return make_geometry(ndim, dims).nseg;
}

vsz_status vsz_dualquant(int ndim, const size_t dims[3], int block_size, int dict_size, const float* d_in,
                         const void* d_consts, uint16_t* d_code, float* d_scratch, uint8_t* d_seg_count,
                         uint64_t* d_hist, void* stream) {
    if (!valid_dims(ndim, dims) || !valid_dict(dict_size) || !d_in || !d_consts || !d_code || !d_scratch ||
        !d_seg_count || !d_hist)
        return VSZ_ERR_INVALID;
    if (!valid_bs(block_size)) return VSZ_ERR_UNSUPPORTED;
    Geometry g = make_geometry(ndim, dims);
    DqArgs a   = make_dq_args(g, block_size, dict_size, d_in, reinterpret_cast<const Consts*>(d_consts), d_code,
                              d_scratch, d_seg_count, reinterpret_cast<unsigned long long*>(d_hist));
    return launch_dq_compress(a, ndim, block_size, S(stream), num_sms());
}

size_t vsz_outlier_gather_tmp_bytes(int ndim, const size_t dims[3]) {
    if (!valid_dims(ndim, dims)) return 0;
    Geometry g = make_geometry(ndim, dims);
    return 256 + 8 * ((g.nseg + 4095) / 4096 + 1) + 256;
}

vsz_status vsz_outlier_gather(int ndim, const size_t dims[3], const uint8_t* d_seg_count, const float* d_scratch,
                              float* d_out, uint64_t* d_count, void* d_tmp, size_t tmp_bytes, void* stream) {
    if (!valid_dims(ndim, dims) || !d_seg_count || !d_scratch || !d_out || !d_count || !d_tmp) return VSZ_ERR_INVALID;
    if (tmp_bytes < vsz_outlier_gather_tmp_bytes(ndim, dims)) return VSZ_ERR_CAPACITY;
    Geometry g = make_geometry(ndim, dims);
    Bump b{reinterpret_cast<uint8_t*>(d_tmp), tmp_bytes};
    GatherArgs ga{};
    ga.status       = b.take<int>(4);
    ga.tile_counter = b.take<uint32_t>(4);
    ga.tile_status  = b.take<unsigned long long>((g.nseg + 4095) / 4096 + 1);
    ga.seg_count    = d_seg_count;
    ga.scratch      = d_scratch;
    ga.nseg         = g.nseg;
    ga.out_f32      = d_out;
    ga.total        = reinterpret_cast<unsigned long long*>(d_count);
    VSZ_CUDA(cudaMemsetAsync(ga.status, 0, sizeof(int), S(stream)));
    return launch_outlier_gather(ga, S(stream));
}

size_t vsz_codebook_bytes(int dict_size) { return (size_t)dict_size * 9 + 64; }
size_t vsz_huff_head_max(int dict_size) { return 8 + tree_bytes_size((uint32_t)(2 * dict_size - 1)); }
size_t vsz_huffman_build_tmp_bytes(int dict_size) { return huff_build_scratch_bytes(dict_size) + 512; }

vsz_status vsz_huffman_build_host(const uint64_t* h_hist, int dict_size, void* h_codebook, uint8_t* h_huff_head,
                                  uint32_t h_info[4]) {
    if (!valid_dict(dict_size) || !h_hist || !h_codebook || !h_huff_head || !h_info) return VSZ_ERR_INVALID;
    uint8_t* cb = static_cast<uint8_t*>(h_codebook);
    int rc = host_huffman_build(h_hist, dict_size, reinterpret_cast<uint64_t*>(cb), cb + 8 * (size_t)dict_size,
                                h_info, h_huff_head);
    return rc ? VSZ_ERR_INVALID : VSZ_OK;
}

int vsz_set_tree_builder(int which) {
    int prev = tree_builder();
    if (which == VSZ_TREE_DEVICE || which == VSZ_TREE_HOST) g_tree_builder.store(which);
    return prev;
}

vsz_status vsz_huffman_build(const uint64_t* d_hist, int dict_size, void* d_codebook, uint8_t* d_huff_head,
                             uint32_t* d_info, void* d_tmp, size_t tmp_bytes, void* stream) {
    if (!valid_dict(dict_size) || !d_hist || !d_codebook || !d_huff_head || !d_info || !d_tmp) return VSZ_ERR_INVALID;
    if (tmp_bytes < vsz_huffman_build_tmp_bytes(dict_size)) return VSZ_ERR_CAPACITY;
    HuffBuildArgs a{};
    a.hist    = reinterpret_cast<const unsigned long long*>(d_hist);
    a.dict    = dict_size;
    a.cb_word = reinterpret_cast<unsigned long long*>(d_codebook);
    a.cb_len  = reinterpret_cast<uint8_t*>(d_codebook) + 8 * (size_t)dict_size;
    a.out     = d_huff_head;
    a.info    = d_info;
    a.status  = reinterpret_cast<int*>(d_tmp);
    a.scratch = reinterpret_cast<uint8_t*>(d_tmp) + 256;
    VSZ_CUDA(cudaMemsetAsync(a.status, 0, sizeof(int), S(stream)));
    return launch_huff_build(a, S(stream));
}

size_t vsz_huffman_encode_tmp_bytes(size_t n) {
    const size_t nc = (n + kChunkSyms - 1) / kChunkSyms;
    Bump b{nullptr, 0};
    b.take<int>(4);
    b.take<uint32_t>(4);
    b.take<unsigned long long>(scan_tmp_tiles(nc) + 1);
    b.take<unsigned long long>(nc + 1);
    b.take<unsigned long long>(2 * nc + 2);
    b.take<uint32_t>(2 * nc + 2);
    b.take<uint16_t>(nc + 8);
    return b.off + 256;
}

vsz_status vsz_huffman_encode(const uint16_t* d_code, size_t n, const void* d_codebook, int dict_size,
                              uint8_t* d_payload, uint64_t* d_bits, uint16_t* d_chunk_bits, void* d_tmp,
                              size_t tmp_bytes, void* stream) {
    if (!valid_dict(dict_size) || !d_code || !d_codebook || !d_payload || !d_bits || !d_tmp) return VSZ_ERR_INVALID;
    if (tmp_bytes < vsz_huffman_encode_tmp_bytes(n)) return VSZ_ERR_CAPACITY;
    Bump b{reinterpret_cast<uint8_t*>(d_tmp), tmp_bytes};
    HuffEncodeArgs a{};
    const size_t nc = (n + kChunkSyms - 1) / kChunkSyms;
    a.status       = b.take<int>(4);
    a.scan_counter = b.take<uint32_t>(4);
    a.scan_status  = b.take<unsigned long long>(scan_tmp_tiles(nc) + 1);
    a.chunk_off    = b.take<unsigned long long>(nc + 1);
    a.edge_idx     = b.take<unsigned long long>(2 * nc + 2);
    a.edge_bits    = b.take<uint32_t>(2 * nc + 2);
    uint16_t* own_chunk_bits = b.take<uint16_t>(nc + 8);  // when the caller wants no index
    a.codes        = d_code;
    a.n            = n;
    a.cb_word      = reinterpret_cast<const unsigned long long*>(d_codebook);
    a.cb_len       = reinterpret_cast<const uint8_t*>(d_codebook) + 8 * (size_t)dict_size;
    a.dict         = dict_size;
    a.out          = d_payload;
    a.total_bits   = reinterpret_cast<unsigned long long*>(d_bits);
    a.chunk_bits   = d_chunk_bits ? d_chunk_bits : own_chunk_bits;
    VSZ_CUDA(cudaMemsetAsync(a.status, 0, sizeof(int), S(stream)));
    return launch_huff_encode(a, S(stream), num_sms());
}

size_t vsz_huffman_decode_tmp_bytes(size_t huff_bytes, size_t n, int dict_size) {
    size_t dims[3] = {n, 1, 1};
    Geometry g = make_geometry(1, dims);
    return layout_decompress(g, dict_size, huff_bytes, 0, 0, nullptr, 0).bytes;
}

vsz_status vsz_huffman_decode(const uint8_t* d_huff, size_t huff_bytes, size_t n, int dict_size, uint16_t* d_code,
                              void* d_tmp, size_t tmp_bytes, void* stream) {
    if (!d_huff || !d_code || !d_tmp || n == 0 || !valid_dict(dict_size) || huff_bytes < 9) return VSZ_ERR_INVALID;
    if (n > 0x7fffffffull) return VSZ_ERR_UNSUPPORTED;
    size_t need = vsz_huffman_decode_tmp_bytes(huff_bytes, n, dict_size);
    if (tmp_bytes < need) return VSZ_ERR_CAPACITY;
    size_t dims[3] = {n, 1, 1};
    Geometry g = make_geometry(1, dims);
    DecompressWs w = layout_decompress(g, dict_size, huff_bytes, 0, 0, reinterpret_cast<uint8_t*>(d_tmp), tmp_bytes);
    // node count / tree size from the big-endian header on the device: copy 4 bytes
    uint8_t h4[4];
    VSZ_CUDA(cudaMemcpyAsync(h4, d_huff, 4, cudaMemcpyDeviceToHost, S(stream)));
    VSZ_CUDA(cudaStreamSynchronize(S(stream)));
    uint32_t nc = ((uint32_t)h4[0] << 24) | ((uint32_t)h4[1] << 16) | ((uint32_t)h4[2] << 8) | h4[3];
    if (nc == 0 || nc > (uint32_t)(2 * dict_size - 1) || 8 + tree_bytes_size(nc) > huff_bytes) return VSZ_ERR_CORRUPT;
    VSZ_CUDA(cudaMemsetAsync(w.status, 0, sizeof(int), S(stream)));
    // decode into w.code, then copy to the caller (w.code is sized for n)
    int rc = decode_codes(d_huff, huff_bytes, nc, tree_bytes_size(nc), n, dict_size, nullptr, 0, 0, w, nullptr,
                          (uint32_t)n, S(stream));
    if (rc) return rc;
    VSZ_CUDA(cudaMemcpyAsync(d_code, w.code, n * sizeof(uint16_t), cudaMemcpyDeviceToDevice, S(stream)));
    int st = 0;
    VSZ_CUDA(cudaMemcpyAsync(&st, w.status, sizeof(int), cudaMemcpyDeviceToHost, S(stream)));
    VSZ_CUDA(cudaStreamSynchronize(S(stream)));
    return st;
}

size_t vsz_dualquant_decompress_tmp_bytes(int ndim, const size_t dims[3]) {
    if (!valid_dims(ndim, dims)) return 0;
    Geometry g = make_geometry(ndim, dims);
    uint32_t nxs = (g.d0 + 255) / 256;
    size_t nsegd = g.nrows * nxs;
    return 1024 + 4 * (nsegd + 64) + 8 * (nsegd + 64) + 8 * (scan_tmp_tiles(nsegd) + 2) + 1024;
}

vsz_status vsz_dualquant_decompress(int ndim, const size_t dims[3], int block_size, int dict_size,
                                    const uint16_t* d_code, const float* d_outliers, uint64_t n_outlier,
                                    const void* d_consts, float* d_out, void* d_tmp, size_t tmp_bytes, void* stream) {
    if (!valid_dims(ndim, dims) || !valid_dict(dict_size) || !d_code || !d_consts || !d_out || !d_tmp)
        return VSZ_ERR_INVALID;
    if (!valid_bs(block_size)) return VSZ_ERR_UNSUPPORTED;
    if (tmp_bytes < vsz_dualquant_decompress_tmp_bytes(ndim, dims)) return VSZ_ERR_CAPACITY;
    Geometry g = make_geometry(ndim, dims);
    uint32_t nxs = (g.d0 + 255) / 256;
    size_t nsegd = g.nrows * nxs;
    Bump b{reinterpret_cast<uint8_t*>(d_tmp), tmp_bytes};
    int* status = b.take<int>(4);
    uint32_t* counter = b.take<uint32_t>(4);
    uint32_t* seg_zero = b.take<uint32_t>(nsegd + 1);
    unsigned long long* seg_off = b.take<unsigned long long>(nsegd + 1);
    unsigned long long* tstat = b.take<unsigned long long>(scan_tmp_tiles(nsegd) + 1);
    VSZ_CUDA(cudaMemsetAsync(status, 0, sizeof(int), S(stream)));
    VSZ_TRY(launch_count_zeros(d_code, g.d0, g.nrows, seg_zero, S(stream), num_sms()));
    VSZ_TRY(launch_scan_u32(seg_zero, seg_off, nsegd, tstat, counter, nullptr, status, S(stream)));
    DqDecArgs a{};
    a.codes      = d_code;
    a.outliers   = d_outliers;
    a.n_outliers = n_outlier;
    a.status     = status;
    a.seg_off    = seg_off;
    a.consts     = reinterpret_cast<const Consts*>(d_consts);
    a.out        = d_out;
    a.d0 = g.d0;
    a.d1 = g.d1;
    a.d2 = g.d2;
    a.n  = g.n;
    a.R  = dict_size / 2;
    bool force_general = getenv("VSZ_FORCE_GENERAL_DECOMPRESS") != nullptr;
    VSZ_TRY(launch_dq_decompress(a, ndim, block_size, force_general, S(stream), num_sms()));
    int st = 0;
    VSZ_CUDA(cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, S(stream)));
    VSZ_CUDA(cudaStreamSynchronize(S(stream)));
    return st;
}

// ---- whole-field compress ------------------------------------------------------------------------

vsz_status vsz_compress_bounds(const vsz_params* p, int ndim, const size_t dims[3], size_t* ws_bytes,
                               size_t* archive_cap) {
    VSZ_TRY(check_params(p, ndim, dims));
    Geometry g = make_geometry(ndim, dims);
    const int nsym = symbol_count(p->dict_size, ndim, p->pad_mode);
    const uint32_t d3[3] = {g.d0, g.d1, g.d2};
    if (ws_bytes) *ws_bytes = layout_compress(g, nsym, nullptr, 0).bytes;
    if (archive_cap) *archive_cap = archive_capacity(g, nsym, pad_count(ndim, d3, p->block_size, p->pad_mode));
    return VSZ_OK;
}

vsz_status vsz_compress(const vsz_params* p, int ndim, const size_t dims[3], const float* d_in, void* d_ws,
                        size_t ws_bytes, uint8_t* d_archive, size_t archive_cap, uint64_t* d_result, void* stream) {
    VSZ_TRY(check_params(p, ndim, dims));
    if (!d_in || !d_ws || !d_archive || !d_result) return VSZ_ERR_INVALID;
    Geometry g   = make_geometry(ndim, dims);
    const int dict = p->dict_size;
    const int nsym = symbol_count(dict, ndim, p->pad_mode);  // histogram / codebook symbols
    const uint32_t d3[3] = {g.d0, g.d1, g.d2};
    const size_t npad    = pad_count(ndim, d3, p->block_size, p->pad_mode);
    CompressWs w = layout_compress(g, nsym, reinterpret_cast<uint8_t*>(d_ws), ws_bytes);
    if (w.bytes > ws_bytes) return VSZ_ERR_CAPACITY;
    if (archive_cap < archive_capacity(g, nsym, npad)) return VSZ_ERR_CAPACITY;
    cudaStream_t st = S(stream);
    const size_t hdr = hdr_bytes(ndim);
    const size_t huff_off = hdr + 4 * npad;  // the Huffman section follows the pad values
    VSZ_CUDA(cudaMemsetAsync(w.status, 0, sizeof(int), st));
    VSZ_CUDA(cudaMemsetAsync(w.hist, 0, sizeof(unsigned long long) * nsym, st));
    VSZ_CUDA(cudaMemsetAsync(w.build_info, 0, 4 * sizeof(uint32_t), st));
    VSZ_CUDA(cudaMemsetAsync(w.total_bits, 0, sizeof(unsigned long long), st));
    VSZ_CUDA(cudaMemsetAsync(w.n_out, 0, sizeof(unsigned long long), st));
    // 1. error-bound family (+ value range for r2r)
    {
        StageTimer t(kStEbSetup, st);
        VSZ_TRY(launch_eb_setup(p->mode, p->eb, d_in, g.n, w.consts, w.mm, st, w.status));
    }
    // 1b. padding (-p): pad values into the archive's pad section (and the global halo value)
    DqArgs a = make_dq_args(g, p->block_size, dict, d_in, w.consts, w.code, w.scratch, w.seg_count, w.hist);
    if (p->pad_mode != VSZ_PAD_NONE) {
        PadArgs pa{};
        pa.x = d_in;
        pa.ndim = ndim;
        pa.bs = p->block_size;
        pa.mode = p->pad_mode;
        pa.type = p->pad_type;
        pa.cst = p->pad_constant;
        pa.d0 = g.d0;
        pa.d1 = g.d1;
        pa.d2 = g.d2;
        pa.nb0 = (g.d0 + p->block_size + 1) / p->block_size;
        pa.nb1 = (g.d1 + p->block_size + 1) / p->block_size;
        pa.nb2 = (g.d2 + p->block_size + 1) / p->block_size;
        pa.consts = w.consts;
        pa.arch = d_archive + hdr;
        pa.halo_g = w.halo_g;
        pa.ws = w.pad_ws;
        VSZ_TRY(launch_pad_values(pa, st, num_sms()));
        const bool global = p->pad_mode == VSZ_PAD_GLOBAL;
        a.pad.vals   = global ? reinterpret_cast<const uint8_t*>(w.halo_g) : d_archive + hdr;
        a.pad.stride = global ? 0 : ((p->pad_mode == VSZ_PAD_EDGE && ndim > 1) ? ndim : 1);
        a.pad.nb0    = pa.nb0;
        a.pad.nb1    = pa.nb1;
        a.dict       = nsym;
        a.smem_hist  = nsym <= 16384 ? 1 : 0;
    }
    // 2. dual-quant + histogram + outlier ranking
    a.strict = (p->flags & VSZ_FLAG_STRICT_EB) ? 1 : 0;
    {
        StageTimer t(kStDualquant, st);
        VSZ_TRY(launch_dq_compress(a, ndim, p->block_size, st, num_sms()));
    }
    // 3. tree + codebook; the Huffman section starts after the header and the pad values
    HuffBuildArgs hb{};
    hb.hist = w.hist;
    hb.dict = nsym;
    hb.hdr_dict = dict;
    hb.cb_word = w.cb_word;
    hb.cb_len = w.cb_len;
    hb.out = d_archive + huff_off;
    hb.info = w.build_info;
    hb.scratch = w.build_scratch;
    hb.status = w.status;
    {
        StageTimer t(kStHuffBuild, st);
        if (tree_builder() == VSZ_TREE_HOST && !stream_capturing(st)) {
            huff_build_prepare();  // a later captured call takes the device builder
            VSZ_TRY(enqueue_host_tree(w.hist, nsym, dict, w.cb_block, d_archive + huff_off, w.status, st));
        } else
            VSZ_TRY(launch_huff_build(hb, st));
    }
    // 4. bitstream, placed after the tree bytes (an offset only the device knows)
    HuffEncodeArgs he{};
    he.codes = w.code;
    he.n = g.n;
    he.cb_word = w.cb_word;
    he.cb_len = w.cb_len;
    he.dict = nsym;
    he.out = d_archive;
    he.out_off = DevOffset{huff_off + 8, w.build_info + 1, nullptr};
    he.total_bits = w.total_bits;
    he.chunk_bits = w.chunk_bits;
    he.chunk_off = w.e_chunk_off;
    he.scan_status = w.e_scan_status;
    he.scan_counter = w.e_counter;
    he.edge_idx = w.e_edge_idx;
    he.edge_bits = w.e_edge_bits;
    he.status = w.status;
    he.build_info = w.build_info;
    VSZ_TRY(launch_huff_encode(he, st, num_sms()));  // stages huff_count, huff_pack
    // 5. outliers after the bitstream, in row-major order
    GatherArgs ga{};
    ga.seg_count = w.seg_count;
    ga.scratch = w.scratch;
    ga.nseg = g.nseg;
    ga.out_bytes = d_archive;
    ga.out_off = DevOffset{huff_off + 8, w.build_info + 1, w.total_bits};
    ga.total = w.n_out;
    ga.tile_status = w.g_tile_status;
    ga.tile_counter = w.g_counter;
    ga.status = w.status;
    ga.seg_off = w.g_seg_off;
    ga.tile_base = w.g_tile_base;
    {
        StageTimer t(kStOutlierGather, st);
        VSZ_TRY(launch_outlier_gather(ga, st, num_sms()));
    }
    // 6. header, result record, trailer with the decode index
    FinalizeArgs f{};
    f.archive = d_archive;
    f.ndim = ndim;
    f.dims[0] = g.d0;
    f.dims[1] = g.d1;
    f.dims[2] = g.d2;
    f.eb = p->eb;
    f.mode = p->mode;
    f.strict = a.strict;
    f.dict = dict;
    f.bs = p->block_size;
    f.hdr = hdr;
    f.npad = npad;
    f.consts = w.consts;
    f.build_info = w.build_info;
    f.payload_bits = w.total_bits;
    f.n_out = w.n_out;
    f.status = w.status;
    f.result = reinterpret_cast<unsigned long long*>(d_result);
    f.chunk_bits = w.chunk_bits;
    f.n_chunks = w.n_chunks;
    int fg = (int)((w.n_chunks + 255) / 256);
    if (fg < 1) fg = 1;
    if (fg > num_sms() * 4) fg = num_sms() * 4;
    {
        StageTimer t(kStFinalize, st);
        k_finalize<<<fg, 256, 0, st>>>(f);
        count_launch();
    }
    VSZ_CUDA(cudaGetLastError());
    return VSZ_OK;
}

// ---- archive parsing (host) ---------------------------------------------------------------------

// The archive as its first head_len bytes and the bytes from data_size on (tail, tail_len of them):
// the header, the Huffman head and the trailer are all the parse reads.
static vsz_status parse_split(const uint8_t* h, size_t head_len, const uint8_t* tail, size_t tail_len, size_t len,
                              vsz_archive_desc* d);

vsz_status vsz_archive_parse(const uint8_t* h, size_t len, vsz_archive_desc* d) {
    if (!h || !d) return VSZ_ERR_INVALID;
    return parse_split(h, len, nullptr, 0, len, d);
}

vsz_status vsz_archive_parse_split(const uint8_t* head, size_t head_len, const uint8_t* tail, size_t tail_len,
                                   vsz_archive_desc* d) {
    if (!head || !d || (!tail && tail_len)) return VSZ_ERR_INVALID;
    return parse_split(head, head_len, tail, tail_len, 0, d);
}

// len == 0: split form (the archive is data_size + tail_len bytes long); else h holds all len bytes
static vsz_status parse_split(const uint8_t* h, size_t head_len, const uint8_t* tail, size_t tail_len, size_t len,
                              vsz_archive_desc* d) {
    memset(d, 0, sizeof(*d));
    const bool split = len == 0;
    if (head_len < 4) return VSZ_ERR_CORRUPT;
    int32_t nd;
    memcpy(&nd, h, 4);
    if (nd < 1 || nd > 3) return VSZ_ERR_CORRUPT;
    size_t hdr = hdr_bytes(nd);
    if (head_len < hdr) return VSZ_ERR_CORRUPT;
    d->ndim = nd;
    d->dims[0] = d->dims[1] = d->dims[2] = 1;
    for (int i = 0; i < nd; i++) {
        int32_t v;
        memcpy(&v, h + 4 * (1 + i), 4);
        if (v <= 0) return VSZ_ERR_CORRUPT;
        d->dims[i] = (uint64_t)v;
    }
    memcpy(&d->eb, h + 4 * (nd + 1), 8);
    uint64_t lens[3];
    memcpy(lens, h + 4 * (nd + 1) + 8, 24);
    d->n_pad = lens[0];
    d->huff_bytes = lens[1];
    d->n_outlier = lens[2];
    d->header_bytes = hdr;
    if (d->n_pad > (1ull << 40) || d->huff_bytes > (1ull << 44) || d->n_outlier > (1ull << 40)) return VSZ_ERR_CORRUPT;
    d->huff_offset = hdr + 4 * d->n_pad;
    d->data_size = d->huff_offset + d->huff_bytes + 4 * d->n_outlier;
    if (split) len = d->data_size + tail_len;
    if (d->data_size > len || d->huff_bytes < 8 || d->huff_offset + 8 > head_len) return VSZ_ERR_CORRUPT;
    const uint8_t* hh = h + d->huff_offset;
    uint32_t nc = ((uint32_t)hh[0] << 24) | ((uint32_t)hh[1] << 16) | ((uint32_t)hh[2] << 8) | hh[3];
    if (nc == 0) return VSZ_ERR_CORRUPT;
    d->node_count = nc;
    d->tree_bytes = tree_bytes_size(nc);
    if (8 + d->tree_bytes > d->huff_bytes) return VSZ_ERR_CORRUPT;
    d->payload_offset = d->huff_offset + 8 + d->tree_bytes;
    d->payload_bytes = d->huff_bytes - 8 - d->tree_bytes;
    d->outlier_offset = d->huff_offset + d->huff_bytes;
    // this library's trailer
    if (len >= d->data_size + kTrailerFixed) {
        const uint8_t* t = split ? tail : h + d->data_size;
        uint32_t u32[4];
        memcpy(u32, t, 16);
        if (u32[0] == kTrailerMagic && u32[1] == kTrailerVersion && u32[2] == kTrailerFixed) {
            d->chunk_syms = u32[3];
            memcpy(&d->eb_final, t + 16, 8);
            memcpy(&d->value_range, t + 24, 8);
            int32_t i32[3];
            memcpy(i32, t + 32, 12);
            d->mode = i32[0] & 0xff;
            d->strict = (i32[0] >> 8) & 1;
            const int f64 = (i32[0] >> 9) & 1;
            d->dict_size = i32[1];
            d->block_size = i32[2];
            uint32_t pad;
            memcpy(&pad, t + 44, 4);
            memcpy(&d->n_chunks, t + 48, 8);
            memcpy(&d->trailer_size, t + 56, 8);
            uint64_t n = d->dims[0] * d->dims[1] * d->dims[2];
            bool ok = d->chunk_syms == (uint32_t)kChunkSyms && d->n_chunks == (n + kChunkSyms - 1) / kChunkSyms &&
                      pad >= kTrailerFixed && d->data_size + pad + 2 * d->n_chunks <= len &&
                      ((d->data_size + pad) % 8) == 0 && valid_dict(d->dict_size) && valid_bs(d->block_size);
            if (f64 && (d->n_outlier & 1)) ok = false;  // 8-byte outliers: an even word count
            if (ok) {
                d->has_trailer = 1;
                d->index_offset = d->data_size + pad;
                d->f64 = f64;
                if (f64) d->n_outlier /= 2;
            }
        }
    }
    return VSZ_OK;
}

static int resolve_decode_params(const vsz_archive_desc* d, const vsz_decompress_opts* o, int* dict, int* bs,
                                 double* ebf) {
    if (d->f64) return VSZ_ERR_UNSUPPORTED;  // vsz_decompress_f64
    if (d->has_trailer) {
        *dict = d->dict_size;
        *bs = d->block_size;
        *ebf = d->eb_final;
    } else {
        if (!o) return VSZ_ERR_INVALID;
        *dict = o->dict_size;
        *bs = o->block_size;
        *ebf = d->eb;
        if (o->mode == VSZ_MODE_R2R) {
            if (!(o->value_range > 0)) return VSZ_ERR_RANGE;
            *ebf = d->eb * o->value_range;  // src/types.cc:58
        }
    }
    if (!valid_dict(*dict)) return VSZ_ERR_INVALID;
    if (!valid_bs(*bs)) return VSZ_ERR_UNSUPPORTED;
    if (!(*ebf > 0)) return VSZ_ERR_INVALID;
    return VSZ_OK;
}

// Symbols a decoder accepts: the dictionary, plus 2 * radius in a padded 1D archive (raw block
// pad values can produce it), while it fits the u16 codes.
static int decode_symbols(const vsz_archive_desc* d, int dict) {
    return (d->ndim == 1 && d->n_pad > 0 && dict < 65536) ? dict + 1 : dict;
}

// How a decompressor reads the pad section (src/vecsz_interface.hh:287-298): one value -> global,
// one per block -> block, ndim per block -> edge; in 2D / 3D any other count means the zero halo,
// in 1D value 0 for every block (src/dualquant.hh:924-927).
static PadView pad_view_of(const vsz_archive_desc* d, int bs, const uint8_t* d_archive) {
    PadView v{};
    if (d->n_pad == 0) return v;
    const uint64_t nb0 = (d->dims[0] + bs + 1) / bs, nb1 = (d->dims[1] + bs + 1) / bs;
    const uint64_t nb = nb0 * nb1 * ((d->dims[2] + bs + 1) / bs);
    v.nb0 = (uint32_t)nb0;
    v.nb1 = (uint32_t)nb1;
    v.vals = d_archive + d->header_bytes;
    if (d->n_pad == 1) v.stride = 0;
    else if (d->n_pad == nb) v.stride = 1;
    else if (d->n_pad == (uint64_t)d->ndim * nb) v.stride = d->ndim == 1 ? 1 : d->ndim;
    else if (d->ndim == 1) v.stride = 0;
    else v.vals = nullptr;
    return v;
}

vsz_status vsz_decompress_bounds(const vsz_archive_desc* d, const vsz_decompress_opts* o, size_t* ws_bytes) {
    if (!d) return VSZ_ERR_INVALID;
    int dict, bs;
    double ebf;
    VSZ_TRY(resolve_decode_params(d, o, &dict, &bs, &ebf));
    size_t dims[3] = {d->dims[0], d->dims[1], d->dims[2]};
    Geometry g = make_geometry(d->ndim, dims);
    if (ws_bytes)
        *ws_bytes = layout_decompress(g, decode_symbols(d, dict), d->payload_bytes, d->n_outlier,
                                      d->has_trailer ? d->n_chunks : 0, nullptr, 0).bytes;
    return VSZ_OK;
}

vsz_status vsz_decompress(const vsz_archive_desc* d, const vsz_decompress_opts* o, const uint8_t* d_archive,
                          void* d_ws, size_t ws_bytes, float* d_out, int* d_status, void* stream) {
    if (!d || !d_archive || !d_ws || !d_out) return VSZ_ERR_INVALID;
    int dict, bs;
    double ebf;
    VSZ_TRY(resolve_decode_params(d, o, &dict, &bs, &ebf));
    size_t dims[3] = {d->dims[0], d->dims[1], d->dims[2]};
    if (!valid_dims(d->ndim, dims)) return VSZ_ERR_CORRUPT;
    Geometry g = make_geometry(d->ndim, dims);
    const int nsym = decode_symbols(d, dict);
    if (d->node_count > (uint32_t)(2 * nsym - 1)) return VSZ_ERR_CORRUPT;
    DecompressWs w = layout_decompress(g, nsym, d->payload_bytes, d->n_outlier, d->has_trailer ? d->n_chunks : 0,
                                       reinterpret_cast<uint8_t*>(d_ws), ws_bytes);
    if (w.bytes > ws_bytes) return VSZ_ERR_CAPACITY;
    cudaStream_t st = S(stream);
    uint32_t nxs = (g.d0 + 255) / 256;
    size_t nsegd = g.nrows * nxs;
    VSZ_CUDA(cudaMemsetAsync(w.status, 0, sizeof(int), st));
    VSZ_CUDA(cudaMemsetAsync(w.seg_zero, 0, 4 * nsegd, st));
    VSZ_TRY(launch_eb_setup(VSZ_MODE_ABS, ebf, nullptr, 0, w.consts, w.mm, st, w.status));
    const uint16_t* idx = d->has_trailer ? reinterpret_cast<const uint16_t*>(d_archive + d->index_offset) : nullptr;
    VSZ_TRY(decode_codes(d_archive + d->huff_offset, d->huff_bytes, d->node_count, d->tree_bytes, g.n, nsym, idx,
                         d->has_trailer ? d->n_chunks : 0, d->chunk_syms, w, idx ? nullptr : w.seg_zero, g.d0, st));
    // outlier ranks: per 512-code chunk from the indexed decoder (block size 8), else per 256-wide
    // row segment
    // VSZ_FORCE_GENERAL_DECOMPRESS: the general reverse-Lorenzo kernel for every block size (tests
    // of that path); it ranks outliers by row segment only
    const bool force_general = getenv("VSZ_FORCE_GENERAL_DECOMPRESS") != nullptr;
    // the block-8 kernel ranks outliers from the decoder's per-chunk zero counts directly, which
    // costs a recount from the chunk start in every row segment holding outliers; with dense
    // outliers (over 1 in 1024 elements) the per-segment zero counts are cheaper
    const bool dense_outliers = d->n_outlier > g.n / 1024;
    const bool chunk_rank     = idx != nullptr && bs == 8 && d->node_count > 1 && !force_general && !dense_outliers;
    // the reverse Lorenzo's arguments (the outlier rank source is set after the zero scan)
    DqDecArgs a{};
    a.codes = w.code;
    a.outliers = w.outliers;
    a.n_outliers = d->n_outlier;
    a.status = w.status;
    a.seg_off = w.seg_off;
    a.chunk_off = chunk_rank ? w.chunk_off : nullptr;
    a.consts = w.consts;
    a.out = d_out;
    a.d0 = g.d0;
    a.d1 = g.d1;
    a.d2 = g.d2;
    a.n = g.n;
    a.R = dict / 2;
    a.strict = d->has_trailer ? d->strict : 0;
    a.xtail  = (g.ndim == 3 && (g.d0 % 8) != 0) ? (g.d0 & ~7u) : g.d0;
    a.pad    = pad_view_of(d, bs, d_archive);
    a.redo   = w.redo;
    a.consts_rw = w.consts;
    a.dq_cache  = w.dq_cache;
    // small 3D fields (the wavefront pass): zeros before each row's x-block of 8
    a.blk_off = w.blk_off;
    const bool blk_rank = bs == 8 && !force_general && d->n_outlier != 0 && dq_w8_applies(a, g.ndim);
    {
        StageTimer t(kStZeroScan, st);
        if (blk_rank) {
            VSZ_TRY(launch_count_zeros_b8(w.code, g.d0, g.nrows, w.blk_zero, st, num_sms()));
            VSZ_TRY(launch_scan_u32(w.blk_zero, w.blk_off, g.nrows * ((g.d0 + 7) / 8), w.scan_status, w.scan_counter,
                                    w.scan_total, w.status, st));
        } else if (chunk_rank) {
            VSZ_TRY(launch_scan_u32(w.chunk_zero, w.chunk_off, d->n_chunks, w.scan_status, w.scan_counter,
                                    w.scan_total, w.status, st));
        } else {
            if (idx) VSZ_TRY(launch_count_zeros(w.code, g.d0, g.nrows, w.seg_zero, st, num_sms()));
            VSZ_TRY(launch_scan_u32(w.seg_zero, w.seg_off, nsegd, w.scan_status, w.scan_counter, w.scan_total,
                                    w.status, st));
        }
        k_check_zeros<<<1, 1, 0, st>>>(w.scan_total, d->n_outlier, w.status);
        count_launch();
    }
    if (d->n_outlier) {
        StageTimer t(kStOutlierCopy, st);
        VSZ_CUDA(cudaMemcpyAsync(w.outliers, d_archive + d->outlier_offset, 4 * d->n_outlier, cudaMemcpyDeviceToDevice,
                                 st));
    }
    a.blk_off = blk_rank ? w.blk_off : nullptr;
    {
        StageTimer t(kStLorenzoDecompress, st);
        VSZ_TRY(launch_dq_decompress(a, d->ndim, bs, force_general, st, num_sms()));
    }
    if (d_status) {
        k_copy_status<<<1, 1, 0, st>>>(w.status, w.consts, d_status);
        count_launch();
    }
    VSZ_CUDA(cudaGetLastError());
    return VSZ_OK;
}

vsz_status vsz_debug_set_spin_limit(long long polls) {
    if (polls <= 0) polls = kSpinLimit;
    VSZ_TRY(set_spin_limit_dq(polls));
    VSZ_TRY(set_spin_limit_huffman(polls));
    return cudaDeviceSynchronize() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

vsz_status vsz_debug_scan_stalled_predecessor(size_t n, int* h_status) { return debug_scan_stalled(n, h_status); }

vsz_status vsz_debug_tree_hold(int hold) {
    tree_worker()->hold.store(hold ? 1 : 0, std::memory_order_relaxed);
    return VSZ_OK;
}

vsz_status vsz_debug_set_tree_wait_ns(long long ns) {
    g_tree_wait_ns.store(ns > 0 ? ns : 2000000000ll, std::memory_order_relaxed);
    return VSZ_OK;
}

}  // extern "C"

// =================================================================================================
// f64 fields (dq_f64.cu): the same pipeline in double precision, error bound guaranteed
// =================================================================================================
namespace {

struct CompressF64Ws {
    Consts* consts;
    unsigned long long* mm;
    int* status;
    unsigned long long* hist;
    long long* s;
    uint16_t* code;
    uint32_t* seg_zero;
    unsigned long long* seg_off;
    unsigned long long* g_scan;
    uint32_t* g_counter;
    unsigned long long* n_out;
    uint8_t* build_scratch;
    uint8_t* cb_block;
    unsigned long long* cb_word;
    uint8_t* cb_len;
    uint32_t* build_info;
    size_t n_chunks;
    unsigned long long* e_chunk_off;
    unsigned long long* e_scan_status;
    unsigned long long* e_edge_idx;
    uint32_t* e_edge_bits;
    uint32_t* e_counter;
    unsigned long long* total_bits;
    uint16_t* chunk_bits;
    size_t bytes;
};

CompressF64Ws layout_compress_f64(const Geometry& g, int dict, uint8_t* base, size_t cap) {
    Bump b{base, cap};
    CompressF64Ws w{};
    const size_t nsegd = g.nrows * ((g.d0 + 255) / 256);
    w.consts    = b.take<Consts>(1);
    w.mm        = b.take<unsigned long long>(2);
    w.status    = b.take<int>(4);
    w.hist      = b.take<unsigned long long>(dict);
    w.s         = b.take<long long>(g.n);
    w.code      = b.take<uint16_t>(g.n + 8);
    w.seg_zero  = b.take<uint32_t>(nsegd + 1);
    w.seg_off   = b.take<unsigned long long>(nsegd + 1);
    w.g_scan    = b.take<unsigned long long>(scan_tmp_tiles(nsegd) + 1);
    w.g_counter = b.take<uint32_t>(4);
    w.n_out     = b.take<unsigned long long>(1);
    w.build_scratch = b.take<uint8_t>(huff_build_scratch_bytes(dict));
    uint8_t* cb  = b.take<uint8_t>(codebook_block_bytes(dict));
    w.cb_block   = cb;
    w.cb_word    = reinterpret_cast<unsigned long long*>(cb);
    w.build_info = cb ? reinterpret_cast<uint32_t*>(cb + 8 * (size_t)dict) : nullptr;
    w.cb_len     = cb ? cb + 8 * (size_t)dict + 16 : nullptr;
    w.n_chunks   = (g.n + kChunkSyms - 1) / kChunkSyms;
    w.e_chunk_off   = b.take<unsigned long long>(w.n_chunks + 1);
    w.e_scan_status = b.take<unsigned long long>(scan_tmp_tiles(w.n_chunks) + 1);
    w.e_edge_idx    = b.take<unsigned long long>(2 * w.n_chunks + 2);
    w.e_edge_bits   = b.take<uint32_t>(2 * w.n_chunks + 2);
    w.e_counter     = b.take<uint32_t>(4);
    w.total_bits    = b.take<unsigned long long>(1);
    w.chunk_bits    = b.take<uint16_t>(w.n_chunks + 8);
    w.bytes         = b.off + 256;
    return w;
}

// the packed block with 8-byte outliers, and the trailer
size_t archive_capacity_f64(const Geometry& g, int dict) { return archive_capacity(g, dict) + 4 * g.n; }

int check_params_f64(const vsz_params* p, int ndim, const size_t dims[3]) {
    VSZ_TRY(check_params(p, ndim, dims));
    // padding keeps the reference's f32 pad section; the f64 path always bounds the error as the
    // strict mode does, so the strict flag changes nothing
    if (p->pad_mode != VSZ_PAD_NONE) return VSZ_ERR_UNSUPPORTED;
    return VSZ_OK;
}

}  // namespace

extern "C" {

vsz_status vsz_compress_f64_bounds(const vsz_params* p, int ndim, const size_t dims[3], size_t* ws_bytes,
                                   size_t* archive_cap) {
    VSZ_TRY(check_params_f64(p, ndim, dims));
    Geometry g = make_geometry(ndim, dims);
    if (ws_bytes) *ws_bytes = layout_compress_f64(g, p->dict_size, nullptr, 0).bytes;
    if (archive_cap) *archive_cap = archive_capacity_f64(g, p->dict_size);
    return VSZ_OK;
}

vsz_status vsz_compress_f64(const vsz_params* p, int ndim, const size_t dims[3], const double* d_in, void* d_ws,
                            size_t ws_bytes, uint8_t* d_archive, size_t archive_cap, uint64_t* d_result,
                            void* stream) {
    VSZ_TRY(check_params_f64(p, ndim, dims));
    if (!d_in || !d_ws || !d_archive || !d_result) return VSZ_ERR_INVALID;
    Geometry g     = make_geometry(ndim, dims);
    const int dict = p->dict_size;
    CompressF64Ws w = layout_compress_f64(g, dict, reinterpret_cast<uint8_t*>(d_ws), ws_bytes);
    if (w.bytes > ws_bytes) return VSZ_ERR_CAPACITY;
    if (archive_cap < archive_capacity_f64(g, dict)) return VSZ_ERR_CAPACITY;
    cudaStream_t st       = S(stream);
    const size_t hdr      = hdr_bytes(ndim);
    const size_t huff_off = hdr;
    VSZ_CUDA(cudaMemsetAsync(w.status, 0, sizeof(int), st));
    VSZ_CUDA(cudaMemsetAsync(w.hist, 0, sizeof(unsigned long long) * dict, st));
    VSZ_CUDA(cudaMemsetAsync(w.build_info, 0, 4 * sizeof(uint32_t), st));
    VSZ_CUDA(cudaMemsetAsync(w.total_bits, 0, sizeof(unsigned long long), st));
    VSZ_CUDA(cudaMemsetAsync(w.n_out, 0, sizeof(unsigned long long), st));
    {
        StageTimer t(kStEbSetup, st);
        VSZ_TRY(launch_eb_setup_f64(p->mode, p->eb, d_in, g.n, w.consts, w.mm, w.status, st, num_sms()));
    }
    F64Args a{};
    a.x       = d_in;
    a.s       = w.s;
    a.code    = w.code;
    a.hist    = w.hist;
    a.consts  = w.consts;
    a.status  = w.status;
    a.n       = g.n;
    a.d0      = g.d0;
    a.d1      = g.d1;
    a.d2      = g.d2;
    a.bs      = p->block_size;
    a.dict    = dict;
    a.archive = d_archive;
    {
        StageTimer t(kStDualquant, st);
        VSZ_TRY(launch_dq_compress_f64(a, ndim, st, num_sms()));
    }
    HuffBuildArgs hb{};
    hb.hist     = w.hist;
    hb.dict     = dict;
    hb.hdr_dict = dict;
    hb.cb_word  = w.cb_word;
    hb.cb_len   = w.cb_len;
    hb.out      = d_archive + huff_off;
    hb.info     = w.build_info;
    hb.scratch  = w.build_scratch;
    hb.status   = w.status;
    {
        StageTimer t(kStHuffBuild, st);
        if (tree_builder() == VSZ_TREE_HOST && !stream_capturing(st)) {
            huff_build_prepare();
            VSZ_TRY(enqueue_host_tree(w.hist, dict, dict, w.cb_block, d_archive + huff_off, w.status, st));
        } else
            VSZ_TRY(launch_huff_build(hb, st));
    }
    HuffEncodeArgs he{};
    he.codes        = w.code;
    he.n            = g.n;
    he.cb_word      = w.cb_word;
    he.cb_len       = w.cb_len;
    he.dict         = dict;
    he.out          = d_archive;
    he.out_off      = DevOffset{huff_off + 8, w.build_info + 1, nullptr};
    he.total_bits   = w.total_bits;
    he.chunk_bits   = w.chunk_bits;
    he.chunk_off    = w.e_chunk_off;
    he.scan_status  = w.e_scan_status;
    he.scan_counter = w.e_counter;
    he.edge_idx     = w.e_edge_idx;
    he.edge_bits    = w.e_edge_bits;
    he.status       = w.status;
    he.build_info   = w.build_info;
    VSZ_TRY(launch_huff_encode(he, st, num_sms()));
    {
        // outliers (code 0) in row-major order after the bitstream: zero codes per 256-wide row
        // segment, their exclusive scan (the total is the outlier count), then the copy
        StageTimer t(kStOutlierGather, st);
        const size_t nsegd = g.nrows * ((g.d0 + 255) / 256);
        VSZ_TRY(launch_count_zeros(w.code, g.d0, g.nrows, w.seg_zero, st, num_sms()));
        VSZ_TRY(launch_scan_u32(w.seg_zero, w.seg_off, nsegd, w.g_scan, w.g_counter, w.n_out, w.status, st));
        VSZ_TRY(launch_gather_f64(a, w.seg_off, DevOffset{huff_off + 8, w.build_info + 1, w.total_bits}, st,
                                  num_sms()));
    }
    FinalizeArgs f{};
    f.archive      = d_archive;
    f.ndim         = ndim;
    f.dims[0]      = g.d0;
    f.dims[1]      = g.d1;
    f.dims[2]      = g.d2;
    f.eb           = p->eb;
    f.mode         = p->mode;
    f.dict         = dict;
    f.bs           = p->block_size;
    f.hdr          = hdr;
    f.consts       = w.consts;
    f.build_info   = w.build_info;
    f.payload_bits = w.total_bits;
    f.n_out        = w.n_out;
    f.status       = w.status;
    f.result       = reinterpret_cast<unsigned long long*>(d_result);
    f.chunk_bits   = w.chunk_bits;
    f.n_chunks     = w.n_chunks;
    f.f64          = 1;
    int fg = (int)((w.n_chunks + 255) / 256);
    if (fg < 1) fg = 1;
    if (fg > num_sms() * 4) fg = num_sms() * 4;
    {
        StageTimer t(kStFinalize, st);
        k_finalize<<<fg, 256, 0, st>>>(f);
        count_launch();
    }
    VSZ_CUDA(cudaGetLastError());
    return VSZ_OK;
}

vsz_status vsz_decompress_f64_bounds(const vsz_archive_desc* d, size_t* ws_bytes) {
    if (!d) return VSZ_ERR_INVALID;
    if (!d->f64 || !d->has_trailer) return VSZ_ERR_UNSUPPORTED;
    size_t dims[3] = {d->dims[0], d->dims[1], d->dims[2]};
    if (!valid_dims(d->ndim, dims) || !valid_dict(d->dict_size) || !valid_bs(d->block_size)) return VSZ_ERR_CORRUPT;
    Geometry g = make_geometry(d->ndim, dims);
    if (ws_bytes) *ws_bytes = layout_decompress(g, d->dict_size, d->payload_bytes, 0, d->n_chunks, nullptr, 0).bytes;
    return VSZ_OK;
}

vsz_status vsz_decompress_f64(const vsz_archive_desc* d, const uint8_t* d_archive, void* d_ws, size_t ws_bytes,
                              double* d_out, int* d_status, void* stream) {
    if (!d || !d_archive || !d_ws || !d_out) return VSZ_ERR_INVALID;
    if (!d->f64 || !d->has_trailer) return VSZ_ERR_UNSUPPORTED;  // f32 archives: vsz_decompress
    size_t dims[3] = {d->dims[0], d->dims[1], d->dims[2]};
    if (!valid_dims(d->ndim, dims) || !valid_dict(d->dict_size) || !valid_bs(d->block_size) || !(d->eb_final > 0))
        return VSZ_ERR_CORRUPT;
    const int dict = d->dict_size;
    if (d->node_count > (uint32_t)(2 * dict - 1)) return VSZ_ERR_CORRUPT;
    Geometry g     = make_geometry(d->ndim, dims);
    DecompressWs w = layout_decompress(g, dict, d->payload_bytes, 0, d->n_chunks, reinterpret_cast<uint8_t*>(d_ws),
                                       ws_bytes);
    if (w.bytes > ws_bytes) return VSZ_ERR_CAPACITY;
    cudaStream_t st    = S(stream);
    const size_t nsegd = g.nrows * ((g.d0 + 255) / 256);
    VSZ_CUDA(cudaMemsetAsync(w.status, 0, sizeof(int), st));
    VSZ_TRY(launch_eb_setup_f64(VSZ_MODE_ABS, d->eb_final, nullptr, 0, w.consts,
                                reinterpret_cast<unsigned long long*>(w.mm), w.status, st, num_sms()));
    const uint16_t* idx = reinterpret_cast<const uint16_t*>(d_archive + d->index_offset);
    VSZ_TRY(decode_codes(d_archive + d->huff_offset, d->huff_bytes, d->node_count, d->tree_bytes, g.n, dict, idx,
                         d->n_chunks, d->chunk_syms, w, nullptr, g.d0, st));
    {
        StageTimer t(kStZeroScan, st);
        VSZ_TRY(launch_count_zeros(w.code, g.d0, g.nrows, w.seg_zero, st, num_sms()));
        VSZ_TRY(launch_scan_u32(w.seg_zero, w.seg_off, nsegd, w.scan_status, w.scan_counter, w.scan_total, w.status,
                                st));
        k_check_zeros<<<1, 1, 0, st>>>(w.scan_total, d->n_outlier, w.status);
        count_launch();
    }
    F64Args a{};
    a.code     = w.code;
    a.consts   = w.consts;
    a.status   = w.status;
    a.n        = g.n;
    a.d0       = g.d0;
    a.d1       = g.d1;
    a.d2       = g.d2;
    a.bs       = d->block_size;
    a.dict     = dict;
    a.outliers = d_archive + d->outlier_offset;
    a.n_out    = d->n_outlier;
    a.out      = d_out;
    {
        StageTimer t(kStLorenzoDecompress, st);
        VSZ_TRY(launch_dq_decompress_f64(a, d->ndim, w.seg_off, st));
    }
    if (d_status) {
        k_copy_status<<<1, 1, 0, st>>>(w.status, w.consts, d_status);
        count_launch();
    }
    VSZ_CUDA(cudaGetLastError());
    return VSZ_OK;
}

// Host buffers: device buffers allocated per call, synchronous.
vsz_status vsz_compress_host_f64(const vsz_params* p, int ndim, const size_t dims[3], const double* h_in,
                                 uint8_t** h_out, size_t* out_bytes, size_t* data_size, size_t* lossless_size,
                                 size_t* n_outlier) {
    if (!p || !h_in || !h_out) return VSZ_ERR_INVALID;
    *h_out = nullptr;
    size_t ws = 0, cap = 0;
    VSZ_TRY(vsz_compress_f64_bounds(p, ndim, dims, &ws, &cap));
    if (p->lossless != VSZ_LOSSLESS_NONE && p->lossless != VSZ_LOSSLESS_ZSTD && p->lossless != VSZ_LOSSLESS_GZIP)
        return VSZ_ERR_UNSUPPORTED;
    const Geometry g = make_geometry(ndim, dims);
    uint8_t *d_in = nullptr, *d_ws = nullptr, *d_arch = nullptr;
    uint64_t* d_res = nullptr;
    std::vector<uint8_t> arch;
    uint64_t res[8] = {};
    int rc = VSZ_ERR_NOMEM;
    if (cudaMalloc(reinterpret_cast<void**>(&d_in), 8 * g.n) == cudaSuccess &&
        cudaMalloc(reinterpret_cast<void**>(&d_ws), ws) == cudaSuccess &&
        cudaMalloc(reinterpret_cast<void**>(&d_arch), cap + 64) == cudaSuccess &&
        cudaMalloc(reinterpret_cast<void**>(&d_res), 64) == cudaSuccess) {
        rc = VSZ_ERR_CUDA;
        if (cudaMemcpy(d_in, h_in, 8 * g.n, cudaMemcpyHostToDevice) == cudaSuccess) {
            rc = vsz_compress_f64(p, ndim, dims, reinterpret_cast<const double*>(d_in), d_ws, ws, d_arch, cap, d_res,
                                  nullptr);
            if (rc == VSZ_OK) rc = cudaMemcpy(res, d_res, 64, cudaMemcpyDeviceToHost) == cudaSuccess ? (int)res[5] : VSZ_ERR_CUDA;
            if (rc == VSZ_OK) {
                arch.resize(res[0] + res[1]);
                if (cudaMemcpy(arch.data(), d_arch, arch.size(), cudaMemcpyDeviceToHost) != cudaSuccess) rc = VSZ_ERR_CUDA;
            }
        }
    }
    cudaFree(d_in);
    cudaFree(d_ws);
    cudaFree(d_arch);
    cudaFree(d_res);
    if (rc != VSZ_OK) return rc;
    size_t ls = 0;
    uint8_t* out = nullptr;
    size_t total = 0;
    if (p->lossless != VSZ_LOSSLESS_NONE) {
        uint8_t* frame = nullptr;
        VSZ_TRY(vsz_lossless_compress(p->lossless, arch.data(), res[0], &frame, &ls));
        total = ls + res[1];
        out   = static_cast<uint8_t*>(malloc(total ? total : 1));
        if (!out) {
            vsz_free_host(frame);
            return VSZ_ERR_NOMEM;
        }
        memcpy(out, frame, ls);
        memcpy(out + ls, arch.data() + res[0], res[1]);  // the trailer follows the frame
        vsz_free_host(frame);
    } else {
        total = arch.size();
        out   = static_cast<uint8_t*>(malloc(total ? total : 1));
        if (!out) return VSZ_ERR_NOMEM;
        memcpy(out, arch.data(), total);
    }
    *h_out = out;
    if (out_bytes) *out_bytes = total;
    if (data_size) *data_size = res[0];
    if (lossless_size) *lossless_size = ls;
    if (n_outlier) *n_outlier = res[2];
    return VSZ_OK;
}

vsz_status vsz_decompress_host_f64(const uint8_t* h_archive, size_t len, size_t data_size, size_t lossless_size,
                                   double** h_out, size_t* n) {
    if (!h_archive || !h_out) return VSZ_ERR_INVALID;
    *h_out = nullptr;
    std::vector<uint8_t> arch;
    if (lossless_size) {  // [frame][trailer]: undo the lossless pass, keep the trailer after the block
        if (lossless_size > len) return VSZ_ERR_CORRUPT;
        uint8_t* block = nullptr;
        size_t blen    = 0;
        VSZ_TRY(vsz_lossless_decompress(h_archive, lossless_size, data_size, &block, &blen));
        arch.assign(block, block + blen);
        vsz_free_host(block);
        arch.insert(arch.end(), h_archive + lossless_size, h_archive + len);
    } else {
        arch.assign(h_archive, h_archive + len);
    }
    vsz_archive_desc d{};
    VSZ_TRY(vsz_archive_parse(arch.data(), arch.size(), &d));
    size_t ws = 0;
    VSZ_TRY(vsz_decompress_f64_bounds(&d, &ws));
    const size_t count = d.dims[0] * d.dims[1] * d.dims[2];
    uint8_t *d_arch = nullptr, *d_ws = nullptr;
    double* d_out = nullptr;
    int* d_st     = nullptr;
    int rc = VSZ_ERR_NOMEM, st = VSZ_OK;
    double* out = static_cast<double*>(malloc(8 * (count ? count : 1)));
    if (out && cudaMalloc(reinterpret_cast<void**>(&d_arch), arch.size() + 64) == cudaSuccess &&
        cudaMalloc(reinterpret_cast<void**>(&d_ws), ws) == cudaSuccess &&
        cudaMalloc(reinterpret_cast<void**>(&d_out), 8 * count) == cudaSuccess &&
        cudaMalloc(reinterpret_cast<void**>(&d_st), 4) == cudaSuccess) {
        rc = VSZ_ERR_CUDA;
        if (cudaMemset(d_arch + arch.size(), 0, 64) == cudaSuccess &&
            cudaMemcpy(d_arch, arch.data(), arch.size(), cudaMemcpyHostToDevice) == cudaSuccess) {
            rc = vsz_decompress_f64(&d, d_arch, d_ws, ws, d_out, d_st, nullptr);
            if (rc == VSZ_OK && (cudaMemcpy(&st, d_st, 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
                                 cudaMemcpy(out, d_out, 8 * count, cudaMemcpyDeviceToHost) != cudaSuccess))
                rc = VSZ_ERR_CUDA;
            if (rc == VSZ_OK) rc = st;
        }
    }
    cudaFree(d_arch);
    cudaFree(d_ws);
    cudaFree(d_out);
    cudaFree(d_st);
    if (rc != VSZ_OK) {
        free(out);
        return rc;
    }
    *h_out = out;
    if (n) *n = count;
    return VSZ_OK;
}

}  // extern "C"
