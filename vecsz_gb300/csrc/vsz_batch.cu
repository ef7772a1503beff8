// Batched compress: many fields of uneven shapes, dimensionalities and error bounds in a handful of
// launches, each over a device-side table of per-field arguments and a list of block-wide tasks
// (one field, a range of its work units).  The plan is built once on the host, where every
// field's geometry is known, and uploaded; vsz_batch_compress then only enqueues device work
// (memsets and launches on the caller's stream), so it can be captured in a CUDA graph.
//
// Per field the result is byte-identical to vsz_compress of that field: the same kernels' unit
// bodies run, only the way units are handed out differs.  The Huffman trees are built on the
// device, one CTA per field, all fields in one launch.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "api_common.cuh"
#include "vsz_device.cuh"
#include "vsz_huffman.h"
#include "vsz_kernels.h"
#include "vsz_profile.h"

using namespace vsz;
using namespace vsz::api;

namespace {

// Per-field control words, one 256-byte record per field, zeroed by one memset.
constexpr size_t kCtlBytes   = 256;
constexpr size_t kCtlConsts  = 0;    // Consts (<= 64 bytes)
constexpr size_t kCtlMm      = 64;   // u32 {max key, min key}
constexpr size_t kCtlStatus  = 72;   // int
constexpr size_t kCtlInfo    = 80;   // u32[4] tree info
constexpr size_t kCtlBits    = 96;   // u64 payload bits
constexpr size_t kCtlNOut    = 104;  // u64 outliers
constexpr size_t kCtlTicket  = 112;  // u32 gather look-back ticket
// after the per-field records: the batch status, then one dual-quant task counter per class
// (dimensionality x block size x aligned or not x tail or not: at most 48)
constexpr size_t kDqNextOff  = 64;
static_assert(kDqNextOff + 4 * 48 <= 256, "the counters fit the control tail");

// Work per task (defaults; vsz_batch_autotune searches the first two): dual-quant warp units,
// encoder chunks, min/max elements.
constexpr uint64_t kDqUnitsPerTask  = 32;
constexpr uint64_t kEncChunksPerTask = 64;
constexpr uint64_t kMinmaxPerTask    = 1 << 20;
constexpr uint64_t kGatherTileSegs   = 4096;  // k_outlier_gather's tile

struct DqGroup {
    int ndim, bs;
    bool vec, tail;
    uint32_t hist_words;
    uint32_t task_off, ntasks;
};

}  // namespace

struct vsz_batch {
    int device = -1;
    int nfields = 0;
    uint8_t* d_tables = nullptr;  // owned: argument tables and task lists
    // device tables
    const MinmaxField* minmax = nullptr;
    const ConstsField* consts = nullptr;
    const DqArgs* dq          = nullptr;
    const HuffBuildArgs* build = nullptr;
    const HuffEncodeArgs* enc  = nullptr;
    const GatherArgs* gather   = nullptr;
    const FinalizeArgs* fin    = nullptr;
    const BatchTask* tasks     = nullptr;
    // launch plan
    uint32_t minmax_off = 0, minmax_n = 0;
    std::vector<DqGroup> dq_groups;
    uint32_t build_smem_n = 0;  // fields [0, build_smem_n) of `build` use the shared-memory builder
    int build_dict_max = 0;
    uint32_t enc_off = 0, enc_n = 0;
    int cb_dict_max = 0;
    uint32_t gather_off = 0, gather_n = 0;
    size_t total_chunks = 0;
    // task lists (own buffer, rebuilt by vsz_batch_set_task_sizes) and what they are built from
    BatchTask* d_tasks = nullptr;
    size_t tasks_cap   = 0;
    uint64_t dq_per = 32, enc_per = 64;
    std::vector<uint64_t> minmax_units, dq_units, enc_units, gather_units;  // per field
    std::vector<std::pair<DqGroup, std::vector<uint32_t>>> classes;
    // workspace regions zeroed per call
    uint8_t* ctl = nullptr;
    size_t ctl_bytes = 0;
    unsigned long long* hist = nullptr;
    size_t hist_bytes = 0;
    unsigned long long* gstatus = nullptr;
    size_t gstatus_bytes = 0;
    uint16_t* all_bits = nullptr;
    unsigned long long* all_off = nullptr;
    unsigned long long* scan_status = nullptr;
    uint32_t* scan_counter = nullptr;
    int* batch_status = nullptr;
};

namespace {

struct FieldGeom {
    Geometry g;
    vsz_params p;
    size_t nch, ntiles;
    bool r2r;
};

// The workspace layout, measured (base == nullptr) or carved.
struct BatchLayout {
    uint8_t* ctl;
    int* batch_status;
    unsigned long long* hist;
    unsigned long long* gstatus;
    uint16_t* all_bits;
    unsigned long long* all_off;
    unsigned long long* scan_status;
    uint32_t* scan_counter;
    std::vector<uint16_t*> code;
    std::vector<uint8_t*> seg_count;
    std::vector<float*> scratch;
    std::vector<uint8_t*> cb;
    std::vector<uint8_t*> build_scratch;
    std::vector<unsigned long long*> edge_idx;
    std::vector<uint32_t*> edge_bits;
    std::vector<size_t> hist_off, gstat_off, chunk_base;
    size_t bytes;
};

BatchLayout layout_batch(const std::vector<FieldGeom>& fg, uint8_t* base, size_t cap) {
    Bump b{base, cap};
    BatchLayout L{};
    const size_t nf = fg.size();
    L.ctl          = b.take<uint8_t>(nf * kCtlBytes + 256);
    L.batch_status = reinterpret_cast<int*>(L.ctl ? L.ctl + nf * kCtlBytes : nullptr);
    size_t hwords = 0, gwords = 0, chunks = 0;
    for (const auto& f : fg) {
        L.hist_off.push_back(hwords);
        hwords += (size_t)f.p.dict_size;
        L.gstat_off.push_back(gwords);
        gwords += f.ntiles + 1;
        L.chunk_base.push_back(chunks);
        chunks += f.nch;
    }
    L.hist         = b.take<unsigned long long>(hwords);
    L.gstatus      = b.take<unsigned long long>(gwords);
    L.all_bits     = b.take<uint16_t>(chunks + 8);
    L.all_off      = b.take<unsigned long long>(chunks + 1);
    L.scan_status  = b.take<unsigned long long>(scan_tmp_tiles(chunks) + 1);
    L.scan_counter = b.take<uint32_t>(4);
    for (const auto& f : fg) {
        L.code.push_back(b.take<uint16_t>(f.g.n + 8));
        L.seg_count.push_back(b.take<uint8_t>(f.g.nseg + 16));
        L.scratch.push_back(b.take<float>(f.g.nseg * kSegX));
        L.cb.push_back(b.take<uint8_t>(codebook_block_bytes(f.p.dict_size)));
        L.build_scratch.push_back(huff_build_in_smem(f.p.dict_size) ? nullptr
                                                                     : b.take<uint8_t>(huff_build_scratch_bytes(f.p.dict_size)));
        L.edge_idx.push_back(b.take<unsigned long long>(2 * f.nch + 2));
        L.edge_bits.push_back(b.take<uint32_t>(2 * f.nch + 2));
    }
    L.bytes = b.off + 256;
    return L;
}

int field_geoms(const vsz_batch_field* fields, int nfields, std::vector<FieldGeom>& out) {
    if (!fields || nfields <= 0) return VSZ_ERR_INVALID;
    out.clear();
    for (int i = 0; i < nfields; i++) {
        const vsz_batch_field& f = fields[i];
        VSZ_TRY(check_params(&f.params, f.ndim, f.dims));
        // strict mode and padding: single-field entry points only
        if ((f.params.flags & VSZ_FLAG_STRICT_EB) || f.params.pad_mode != VSZ_PAD_NONE) return VSZ_ERR_UNSUPPORTED;
        FieldGeom fg{};
        fg.g      = make_geometry(f.ndim, f.dims);
        fg.p      = f.params;
        fg.nch    = (fg.g.n + kChunkSyms - 1) / kChunkSyms;
        fg.ntiles = (fg.g.nseg + kGatherTileSegs - 1) / kGatherTileSegs;
        fg.r2r    = f.params.mode == VSZ_MODE_R2R;
        out.push_back(fg);
    }
    return VSZ_OK;
}

void add_tasks(std::vector<BatchTask>& t, uint32_t field, uint64_t units, uint64_t per) {
    for (uint64_t u = 0; u < units; u += per) {
        BatchTask k{};
        k.u0    = u;
        k.u1    = std::min(units, u + per);
        k.field = field;
        t.push_back(k);
    }
}

// Header, result record and trailer of every field: one block per field.
__global__ void __launch_bounds__(256) k_finalize_batch(const FinalizeArgs* __restrict__ args, uint32_t nfields) {
    for (uint32_t f = blockIdx.x; f < nfields; f += gridDim.x) finalize_field(args[f], 0, 1);
}

int launch_finalize_batch(const FinalizeArgs* args, uint32_t nfields, cudaStream_t st, int num_sms) {
    if (nfields == 0) return VSZ_OK;
    const uint32_t grid = nfields < (uint32_t)num_sms * 8 ? nfields : (uint32_t)num_sms * 8;
    k_finalize_batch<<<grid, 256, 0, st>>>(args, nfields);
    count_launch();
    return cudaGetLastError() == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

// Task lists from the per-field unit counts at the batch's task sizes, uploaded (synchronous).
int upload_tasks(vsz_batch* B) {
    std::vector<BatchTask> tasks;
    const uint32_t nf = (uint32_t)B->nfields;
    B->minmax_off = 0;
    for (uint32_t f = 0; f < nf; f++)
        if (B->minmax_units[f]) add_tasks(tasks, f, B->minmax_units[f], kMinmaxPerTask);
    B->minmax_n = (uint32_t)tasks.size();
    B->dq_groups.clear();
    for (auto& kv : B->classes) {
        DqGroup grp  = kv.first;
        grp.task_off = (uint32_t)tasks.size();
        for (uint32_t f : kv.second) add_tasks(tasks, f, B->dq_units[f], B->dq_per);
        grp.ntasks = (uint32_t)tasks.size() - grp.task_off;
        B->dq_groups.push_back(grp);
    }
    B->enc_off = (uint32_t)tasks.size();
    for (uint32_t f = 0; f < nf; f++) add_tasks(tasks, f, B->enc_units[f], B->enc_per);
    B->enc_n      = (uint32_t)tasks.size() - B->enc_off;
    B->gather_off = (uint32_t)tasks.size();
    for (uint32_t f = 0; f < nf; f++) add_tasks(tasks, f, B->gather_units[f], 1);
    B->gather_n = (uint32_t)tasks.size() - B->gather_off;
    if (tasks.size() > B->tasks_cap) {
        if (B->d_tasks) cudaFree(B->d_tasks);
        B->d_tasks   = nullptr;
        B->tasks_cap = 0;
        if (cudaMalloc(reinterpret_cast<void**>(&B->d_tasks), sizeof(BatchTask) * tasks.size()) != cudaSuccess)
            return VSZ_ERR_NOMEM;
        B->tasks_cap = tasks.size();
    }
    if (cudaMemcpy(B->d_tasks, tasks.data(), sizeof(BatchTask) * tasks.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return VSZ_ERR_CUDA;
    B->tasks = B->d_tasks;
    return VSZ_OK;
}

}  // namespace

extern "C" {

vsz_status vsz_batch_workspace_bytes(const vsz_batch_field* fields, int nfields, size_t* ws_bytes) {
    std::vector<FieldGeom> fg;
    VSZ_TRY(field_geoms(fields, nfields, fg));
    if (ws_bytes) *ws_bytes = layout_batch(fg, nullptr, 0).bytes;
    return VSZ_OK;
}

vsz_status vsz_batch_create(const vsz_batch_field* fields, int nfields, void* d_ws, size_t ws_bytes, uint64_t* d_results,
                            vsz_batch** out) {
    if (!out || !d_ws || !d_results) return VSZ_ERR_INVALID;
    *out = nullptr;
    std::vector<FieldGeom> fg;
    VSZ_TRY(field_geoms(fields, nfields, fg));
    BatchLayout L = layout_batch(fg, reinterpret_cast<uint8_t*>(d_ws), ws_bytes);
    if (L.bytes > ws_bytes) return VSZ_ERR_CAPACITY;
    for (int i = 0; i < nfields; i++) {
        if (!fields[i].d_in || !fields[i].d_archive) return VSZ_ERR_INVALID;
        if (fields[i].archive_capacity < archive_capacity(fg[i].g, fg[i].p.dict_size)) return VSZ_ERR_CAPACITY;
    }
    const uint32_t nf = (uint32_t)nfields;
    std::vector<MinmaxField> mm(nf);
    std::vector<ConstsField> cs(nf);
    std::vector<DqArgs> dq(nf);
    std::vector<HuffEncodeArgs> enc(nf);
    std::vector<GatherArgs> ga(nf);
    std::vector<FinalizeArgs> fin(nf);
    std::vector<HuffBuildArgs> build_smem, build_glob;
    vsz_batch* B = new vsz_batch();
    B->nfields   = nfields;
    cudaGetDevice(&B->device);
    // ---- per-field argument tables
    for (uint32_t f = 0; f < nf; f++) {
        const vsz_batch_field& F = fields[f];
        const FieldGeom& G       = fg[f];
        const int dict           = G.p.dict_size;
        uint8_t* ctl             = L.ctl + (size_t)f * kCtlBytes;
        Consts* consts           = reinterpret_cast<Consts*>(ctl + kCtlConsts);
        uint32_t* mmw            = reinterpret_cast<uint32_t*>(ctl + kCtlMm);
        int* status              = reinterpret_cast<int*>(ctl + kCtlStatus);
        uint32_t* info           = reinterpret_cast<uint32_t*>(ctl + kCtlInfo);
        unsigned long long* bits = reinterpret_cast<unsigned long long*>(ctl + kCtlBits);
        unsigned long long* nout = reinterpret_cast<unsigned long long*>(ctl + kCtlNOut);
        uint32_t* ticket         = reinterpret_cast<uint32_t*>(ctl + kCtlTicket);
        unsigned long long* hist = L.hist + L.hist_off[f];
        const size_t hdr         = hdr_bytes(G.g.ndim);
        uint8_t* cb              = L.cb[f];
        auto* cb_word            = reinterpret_cast<unsigned long long*>(cb);
        uint8_t* cb_len          = cb + 8 * (size_t)dict + 16;

        mm[f] = MinmaxField{F.d_in, mmw};
        cs[f] = ConstsField{G.p.mode, G.p.eb, mmw, F.d_in, consts, status};
        dq[f] = make_dq_args(G.g, G.p.block_size, dict, F.d_in, consts, L.code[f], L.scratch[f], L.seg_count[f], hist);

        HuffBuildArgs hb{};
        hb.hist    = hist;
        hb.dict    = dict;
        hb.cb_word = cb_word;
        hb.cb_len  = cb_len;
        hb.out     = F.d_archive + hdr;
        hb.info    = info;
        hb.scratch = L.build_scratch[f];
        hb.status  = status;
        if (huff_build_in_smem(dict)) {
            hb.ws_in_smem = 1;
            build_smem.push_back(hb);
            B->build_dict_max = std::max(B->build_dict_max, dict);
        } else {
            hb.ws_in_smem = 0;
            build_glob.push_back(hb);
        }

        HuffEncodeArgs& he = enc[f];
        he            = HuffEncodeArgs{};
        he.codes      = L.code[f];
        he.n          = G.g.n;
        he.cb_word    = cb_word;
        he.cb_len     = cb_len;
        he.dict       = dict;
        he.out        = F.d_archive;
        he.out_off    = DevOffset{hdr + 8, info + 1, nullptr};
        he.total_bits = bits;
        he.chunk_bits = L.all_bits + L.chunk_base[f];
        he.chunk_off  = L.all_off + L.chunk_base[f];
        he.edge_idx   = L.edge_idx[f];
        he.edge_bits  = L.edge_bits[f];
        he.status     = status;
        he.build_info = info;
        huff_encode_prepare(he);
        if (he.cb_in_smem) B->cb_dict_max = std::max(B->cb_dict_max, dict);

        GatherArgs& g = ga[f];
        g             = GatherArgs{};
        g.seg_count   = L.seg_count[f];
        g.scratch     = L.scratch[f];
        g.nseg        = G.g.nseg;
        g.out_bytes   = F.d_archive;
        g.out_off     = DevOffset{hdr + 8, info + 1, bits};
        g.total       = nout;
        g.tile_status = L.gstatus + L.gstat_off[f];
        g.tile_counter = ticket;
        g.status      = status;
        g.ntiles      = (uint32_t)G.ntiles;

        FinalizeArgs& fa = fin[f];
        fa               = FinalizeArgs{};
        fa.archive       = F.d_archive;
        fa.ndim          = G.g.ndim;
        fa.dims[0]       = G.g.d0;
        fa.dims[1]       = G.g.d1;
        fa.dims[2]       = G.g.d2;
        fa.eb            = G.p.eb;
        fa.mode          = G.p.mode;
        fa.dict          = dict;
        fa.bs            = G.p.block_size;
        fa.hdr           = hdr;
        fa.consts        = consts;
        fa.build_info    = info;
        fa.payload_bits  = bits;
        fa.n_out         = nout;
        fa.status        = status;
        fa.result        = reinterpret_cast<unsigned long long*>(d_results) + 8 * (size_t)f;
        fa.chunk_bits    = he.chunk_bits;
        fa.n_chunks      = G.nch;
    }
    // ---- what the task lists are built from
    for (uint32_t f = 0; f < nf; f++) {
        B->minmax_units.push_back(fg[f].r2r ? fg[f].g.n : 0);
        B->dq_units.push_back(dq[f].nunits);
        B->enc_units.push_back(fg[f].nch);
        B->gather_units.push_back(fg[f].ntiles);
    }
    std::map<std::tuple<int, int, bool, bool>, std::vector<uint32_t>> classes;
    for (uint32_t f = 0; f < nf; f++) {
        const FieldGeom& G = fg[f];
        const bool vec     = (G.g.d0 % 4 == 0) && ((reinterpret_cast<uintptr_t>(fields[f].d_in) & 15u) == 0);
        const bool tail    = G.g.ndim >= 2 && (G.g.d0 % 8) != 0;
        classes[std::make_tuple(G.g.ndim, G.p.block_size, vec, tail)].push_back(f);
    }
    for (auto& kv : classes) {
        DqGroup grp{};
        std::tie(grp.ndim, grp.bs, grp.vec, grp.tail) = kv.first;
        for (uint32_t f : kv.second)
            if (dq[f].smem_hist) grp.hist_words = std::max(grp.hist_words, (uint32_t)((dq[f].dict + 3) & ~3));
        B->classes.emplace_back(grp, kv.second);
    }
    B->dq_per  = kDqUnitsPerTask;
    B->enc_per = kEncChunksPerTask;
    B->total_chunks = L.chunk_base.empty() ? 0 : L.chunk_base.back() + fg.back().nch;
    // ---- upload
    std::vector<HuffBuildArgs> build = build_smem;
    build.insert(build.end(), build_glob.begin(), build_glob.end());
    B->build_smem_n = (uint32_t)build_smem.size();
    size_t off = 0;
    auto place = [&](size_t bytes) {
        off = (off + 255) & ~(size_t)255;
        size_t at = off;
        off += bytes;
        return at;
    };
    const size_t o_mm = place(sizeof(MinmaxField) * nf), o_cs = place(sizeof(ConstsField) * nf),
                 o_dq = place(sizeof(DqArgs) * nf), o_bd = place(sizeof(HuffBuildArgs) * nf),
                 o_en = place(sizeof(HuffEncodeArgs) * nf), o_ga = place(sizeof(GatherArgs) * nf),
                 o_fi = place(sizeof(FinalizeArgs) * nf);
    const size_t table_bytes = off + 256;
    std::vector<uint8_t> h(table_bytes, 0);
    memcpy(h.data() + o_mm, mm.data(), sizeof(MinmaxField) * nf);
    memcpy(h.data() + o_cs, cs.data(), sizeof(ConstsField) * nf);
    memcpy(h.data() + o_dq, dq.data(), sizeof(DqArgs) * nf);
    memcpy(h.data() + o_bd, build.data(), sizeof(HuffBuildArgs) * nf);
    memcpy(h.data() + o_en, enc.data(), sizeof(HuffEncodeArgs) * nf);
    memcpy(h.data() + o_ga, ga.data(), sizeof(GatherArgs) * nf);
    memcpy(h.data() + o_fi, fin.data(), sizeof(FinalizeArgs) * nf);
    if (cudaMalloc(reinterpret_cast<void**>(&B->d_tables), table_bytes) != cudaSuccess) {
        delete B;
        return VSZ_ERR_NOMEM;
    }
    if (cudaMemcpy(B->d_tables, h.data(), table_bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(B->d_tables);
        delete B;
        return VSZ_ERR_CUDA;
    }
    B->minmax = reinterpret_cast<const MinmaxField*>(B->d_tables + o_mm);
    B->consts = reinterpret_cast<const ConstsField*>(B->d_tables + o_cs);
    B->dq     = reinterpret_cast<const DqArgs*>(B->d_tables + o_dq);
    B->build  = reinterpret_cast<const HuffBuildArgs*>(B->d_tables + o_bd);
    B->enc    = reinterpret_cast<const HuffEncodeArgs*>(B->d_tables + o_en);
    B->gather = reinterpret_cast<const GatherArgs*>(B->d_tables + o_ga);
    B->fin    = reinterpret_cast<const FinalizeArgs*>(B->d_tables + o_fi);
    B->ctl           = L.ctl;
    B->ctl_bytes     = (size_t)nf * kCtlBytes + 256;
    B->batch_status  = L.batch_status;
    B->hist          = L.hist;
    B->hist_bytes    = 0;
    for (uint32_t f = 0; f < nf; f++) B->hist_bytes += 8 * (size_t)fg[f].p.dict_size;
    B->gstatus       = L.gstatus;
    B->gstatus_bytes = 0;
    for (uint32_t f = 0; f < nf; f++) B->gstatus_bytes += 8 * (fg[f].ntiles + 1);
    B->all_bits     = L.all_bits;
    B->all_off      = L.all_off;
    B->scan_status  = L.scan_status;
    B->scan_counter = L.scan_counter;
    const int rc    = upload_tasks(B);
    if (rc != VSZ_OK) {
        vsz_batch_destroy(B);
        return rc;
    }
    *out = B;
    return VSZ_OK;
}

vsz_status vsz_batch_set_task_sizes(vsz_batch* B, int dq_units, int enc_chunks) {
    if (!B || dq_units < 1 || enc_chunks < 1) return VSZ_ERR_INVALID;
    B->dq_per  = (uint64_t)dq_units;
    B->enc_per = (uint64_t)enc_chunks;
    return upload_tasks(B);
}

vsz_status vsz_batch_autotune(vsz_batch* B, int iterations, int* best_dq_units, int* best_enc_chunks, void* stream) {
    if (!B || iterations < 1) return VSZ_ERR_INVALID;
    cudaStream_t st = S(stream);
    cudaEvent_t e0, e1;
    VSZ_CUDA(cudaEventCreate(&e0));
    VSZ_CUDA(cudaEventCreate(&e1));
    auto time_cfg = [&](uint64_t dq, uint64_t enc, float* ms) -> int {
        VSZ_TRY(vsz_batch_set_task_sizes(B, (int)dq, (int)enc));
        VSZ_TRY(vsz_batch_compress(B, stream));  // warm-up
        VSZ_CUDA(cudaEventRecord(e0, st));
        for (int i = 0; i < iterations; i++) VSZ_TRY(vsz_batch_compress(B, stream));
        VSZ_CUDA(cudaEventRecord(e1, st));
        VSZ_CUDA(cudaEventSynchronize(e1));
        VSZ_CUDA(cudaEventElapsedTime(ms, e0, e1));
        return VSZ_OK;
    };
    // coordinate search: dual-quant task size first, then the encoder's
    static const uint64_t kDq[]  = {8, 16, 32, 64, 128};
    static const uint64_t kEnc[] = {16, 32, 64, 128, 256};
    uint64_t bdq = B->dq_per, benc = B->enc_per;
    float best = 3.4e38f, ms = 0.f;
    int rc = VSZ_OK;
    for (uint64_t dq : kDq) {
        if ((rc = time_cfg(dq, benc, &ms)) != VSZ_OK) break;
        if (ms < best) {
            best = ms;
            bdq  = dq;
        }
    }
    best = 3.4e38f;
    for (uint64_t enc : kEnc) {
        if (rc != VSZ_OK || (rc = time_cfg(bdq, enc, &ms)) != VSZ_OK) break;
        if (ms < best) {
            best = ms;
            benc = enc;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != VSZ_OK) return rc;
    if (best_dq_units) *best_dq_units = (int)bdq;
    if (best_enc_chunks) *best_enc_chunks = (int)benc;
    return vsz_batch_set_task_sizes(B, (int)bdq, (int)benc);
}

vsz_status vsz_batch_compress(vsz_batch* B, void* stream) {
    if (!B) return VSZ_ERR_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != B->device) return VSZ_ERR_INVALID;
    cudaStream_t st = S(stream);
    const int sms   = num_sms();
    const uint32_t nf = (uint32_t)B->nfields;
    // control words (status, tree info, sizes, tickets, the batch status) to zero, the min key
    // of every field to 0xffffffff; histograms and look-back status to zero
    VSZ_CUDA(cudaMemsetAsync(B->ctl, 0, B->ctl_bytes, st));
    VSZ_CUDA(cudaMemset2DAsync(B->ctl + kCtlMm + 4, kCtlBytes, 0xff, 4, nf, st));
    VSZ_CUDA(cudaMemsetAsync(B->hist, 0, B->hist_bytes, st));
    VSZ_CUDA(cudaMemsetAsync(B->gstatus, 0, B->gstatus_bytes, st));
    {
        StageTimer t(kStEbSetup, st);
        VSZ_TRY(launch_minmax_batch(B->minmax, B->tasks + B->minmax_off, B->minmax_n, st, sms));
        VSZ_TRY(launch_consts_batch(B->consts, nf, st));
    }
    {
        StageTimer t(kStDualquant, st);
        uint32_t* next = reinterpret_cast<uint32_t*>(B->ctl + (size_t)nf * kCtlBytes + kDqNextOff);
        for (size_t i = 0; i < B->dq_groups.size(); i++) {
            const DqGroup& g = B->dq_groups[i];
            VSZ_TRY(launch_dq_compress_batch(B->dq, B->tasks + g.task_off, g.ntasks, g.ndim, g.bs, g.vec, g.tail,
                                             g.hist_words, next + i, st, sms));
        }
    }
    {
        StageTimer t(kStHuffBuild, st);
        huff_build_prepare();
        VSZ_TRY(launch_huff_build_batch(B->build, B->build_smem_n, true, B->build_dict_max, st, sms));
        VSZ_TRY(launch_huff_build_batch(B->build + B->build_smem_n, nf - B->build_smem_n, false, 0, st, sms));
    }
    VSZ_TRY(launch_huff_encode_batch(B->enc, nf, B->tasks + B->enc_off, B->enc_n, B->cb_dict_max, B->all_bits,
                                     B->all_off, B->total_chunks, B->scan_status, B->scan_counter, B->batch_status,
                                     st, sms));
    {
        StageTimer t(kStOutlierGather, st);
        VSZ_TRY(launch_outlier_gather_batch(B->gather, B->tasks + B->gather_off, B->gather_n, st, sms));
    }
    {
        StageTimer t(kStFinalize, st);
        VSZ_TRY(launch_finalize_batch(B->fin, nf, st, sms));
    }
    VSZ_CUDA(cudaGetLastError());
    return VSZ_OK;
}

void vsz_batch_destroy(vsz_batch* B) {
    if (!B) return;
    if (B->d_tables) cudaFree(B->d_tables);
    if (B->d_tasks) cudaFree(B->d_tasks);
    delete B;
}

}  // extern "C"
