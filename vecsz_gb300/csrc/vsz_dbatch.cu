// Batched decompress: many archives of uneven shapes, dimensionalities and error bounds in a handful
// of launches, each over a device-side table of per-field arguments and a list of block-wide tasks
// (one field, a range of its work units) -- the decompress side of vsz_batch.cu.  The plan is built
// once on the host from the parsed archives and uploaded; vsz_dbatch_decompress then only enqueues
// device work (memsets and launches on the caller's stream), so it can be captured in a CUDA graph.
//
// Per field the output is bit-identical to vsz_decompress of that archive: the same kernels' unit
// bodies run (Huffman tables, the indexed decoders, the block-8 reverse Lorenzo and its separable
// pass), only the way units are handed out differs.  Both chunk-index scans (bits per chunk, zero
// codes per chunk) run once over all fields' chunks; each field reads its offsets relative to its
// first chunk.
//
// Replaces, per field: Decompress (src/vecsz_interface.hh:232-374) -- decode_withTree
// (src/huffman.hh:679-691), the outlier scatter (:313-317) and x_lorenzo_{1,2,3}d1l
// (src/dualquant.hh:915-1043).
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

// Per-field control words, one 128-byte record per field, zeroed by one memset per call.
constexpr size_t kDCtlBytes  = 128;
constexpr size_t kDCtlConsts = 0;   // Consts (<= 64 bytes)
constexpr size_t kDCtlStatus = 64;  // int
constexpr size_t kDCtlInfo   = 80;  // u32[4] tree info (k_huff_table)

constexpr uint64_t kDecTaskChunks = 256;      // one decoder CTA: lane t decodes chunk u0 + t
constexpr uint64_t kCopyTaskBytes = 1 << 18;  // index and outlier copies
constexpr uint64_t kDqTaskUnits   = 1;        // reverse-Lorenzo warp units per task (one warp's)
constexpr size_t kDqNextOff       = 64;       // after the batch status in the control tail: one
constexpr size_t kDqMaxClasses    = 16;       // task counter per reverse-Lorenzo class

// A byte range copied into an aligned buffer (the archive's index and outlier sections).
struct DCopy {
    const uint8_t* src;
    uint8_t* dst;
    const int* status;
};

// Per-field bookkeeping after the decode: zero codes against the archive's outlier count, and the
// field's final status.
struct DCheck {
    const unsigned long long* zoff;  // the field's first entry of the zero-count scan
    unsigned long long nch;          // its chunks (zoff[nch] - zoff[0] = its zero codes)
    unsigned long long n_out;
    const Consts* consts;
    int* status;
    int* out_status;                 // caller's status array entry
    uint32_t* redo;                  // separable pass: count word to clear, or null
};

struct DField {
    Geometry g;
    int nsym;
    double ebf;
    size_t nch;
    size_t units;  // block-8 warp units
    bool sep, vec, konst;
};

struct DqClass {
    int ndim;
    bool vec, sep;
    uint32_t task_off, ntasks;
};

__global__ void k_dbatch_init(const DCheck* __restrict__ c, uint32_t nfields) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < nfields && c[f].redo) c[f].redo[0] = 0u;
}

// Bytes [u0, u1) of copy `field`: whole aligned words when source and destination allow.
__global__ void __launch_bounds__(256) k_dbatch_copy(const DCopy* __restrict__ cp, const BatchTask* __restrict__ tasks,
                                                     uint32_t ntasks) {
    for (uint32_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
        const BatchTask tk = tasks[t];
        const DCopy c      = cp[tk.field];
        if (*c.status != VSZ_OK) continue;
        const bool words = ((reinterpret_cast<uintptr_t>(c.src) | reinterpret_cast<uintptr_t>(c.dst) | tk.u0 | tk.u1) & 3u) == 0;
        if (words) {
            const uint32_t* s = reinterpret_cast<const uint32_t*>(c.src);
            uint32_t* d       = reinterpret_cast<uint32_t*>(c.dst);
            for (size_t i = tk.u0 / 4 + threadIdx.x; i < tk.u1 / 4; i += blockDim.x) d[i] = s[i];
        } else {
            for (size_t i = tk.u0 + threadIdx.x; i < tk.u1; i += blockDim.x) c.dst[i] = c.src[i];
        }
    }
}

// A field's zero codes must equal its outlier count; a failed scan fails every field.
__global__ void k_dbatch_check(const DCheck* __restrict__ c, uint32_t nfields, const int* scan_status) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nfields) return;
    const DCheck k = c[f];
    if (*scan_status != VSZ_OK) set_status(k.status, *scan_status);
    if (k.zoff[k.nch] - k.zoff[0] != k.n_out) set_status(k.status, VSZ_ERR_CORRUPT);
}

__global__ void k_dbatch_status(const DCheck* __restrict__ c, uint32_t nfields) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nfields) return;
    const DCheck k = c[f];
    *k.out_status  = k.consts->status != VSZ_OK ? k.consts->status : *k.status;
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

int field_of(const vsz_dbatch_field& F, DField& out) {
    const vsz_archive_desc& d = F.desc;
    if (!F.d_archive || !F.d_out) return VSZ_ERR_INVALID;
    size_t dims[3] = {(size_t)d.dims[0], (size_t)d.dims[1], (size_t)d.dims[2]};
    if (!valid_dims(d.ndim, dims)) return VSZ_ERR_CORRUPT;
    // the batch needs this library's index (trailer) and the block-8 kernels; padded and strict
    // archives go through vsz_decompress
    if (!d.has_trailer || d.chunk_syms != (uint32_t)kChunkSyms) return VSZ_ERR_UNSUPPORTED;
    if (d.block_size != 8 || d.n_pad != 0 || d.strict || d.f64) return VSZ_ERR_UNSUPPORTED;
    if (!valid_dict(d.dict_size) || !(d.eb_final > 0)) return VSZ_ERR_CORRUPT;
    out.g    = make_geometry(d.ndim, dims);
    out.nsym = d.dict_size;
    if (d.node_count == 0 || d.node_count > (uint32_t)(2 * out.nsym - 1)) return VSZ_ERR_CORRUPT;
    out.ebf   = d.eb_final;
    out.nch   = (out.g.n + kChunkSyms - 1) / kChunkSyms;
    if (d.n_chunks != out.nch) return VSZ_ERR_CORRUPT;
    out.konst = d.node_count == 1;
    DqDecArgs a{};
    a.d0 = out.g.d0;
    a.d1 = out.g.d1;
    a.d2 = out.g.d2;
    dq_b8_geometry(a, d.ndim);
    out.units = a.nunits;
    return VSZ_OK;
}

struct DLayout {
    uint8_t* ctl;
    int* batch_status;
    uint16_t* all_bits;
    unsigned long long *all_start, *all_zoff;
    uint32_t* all_zero;
    unsigned long long* scan_status;
    uint32_t* scan_counter;
    std::vector<uint32_t*> table, table2, child, node_sym, parent, walk, redo;
    std::vector<uint16_t*> code;
    std::vector<float*> outliers;
    std::vector<size_t> chunk_base;
    size_t bytes;
};

DLayout layout_dbatch(const std::vector<DField>& fs, const vsz_dbatch_field* fields, uint8_t* base, size_t cap) {
    Bump b{base, cap};
    DLayout L{};
    const size_t nf = fs.size();
    L.ctl          = b.take<uint8_t>(nf * kDCtlBytes + 256);
    L.batch_status = reinterpret_cast<int*>(L.ctl ? L.ctl + nf * kDCtlBytes : nullptr);
    size_t T = 0;
    for (const auto& f : fs) {
        L.chunk_base.push_back(T);
        T += f.nch;
    }
    L.all_bits     = b.take<uint16_t>(T + 8);
    L.all_start    = b.take<unsigned long long>(T + 1);
    L.all_zero     = b.take<uint32_t>(T + 1);
    L.all_zoff     = b.take<unsigned long long>(T + 1);
    L.scan_status  = b.take<unsigned long long>(scan_tmp_tiles(T) + 1);
    L.scan_counter = b.take<uint32_t>(4);
    for (size_t i = 0; i < nf; i++) {
        const DField& f     = fs[i];
        const uint32_t maxn = (uint32_t)(2 * f.nsym);
        L.table.push_back(b.take<uint32_t>(1u << kDecBits));
        L.table2.push_back(b.take<uint32_t>(table2_capacity(maxn - 1)));
        L.child.push_back(b.take<uint32_t>(2 * (size_t)maxn));
        L.node_sym.push_back(b.take<uint32_t>(maxn));
        L.parent.push_back(b.take<uint32_t>(maxn));
        L.walk.push_back(b.take<uint32_t>(maxn));
        L.code.push_back(b.take<uint16_t>(f.g.n + 8));
        L.outliers.push_back(b.take<float>(fields[i].desc.n_outlier + 4));
        L.redo.push_back(f.sep ? b.take<uint32_t>(f.units + 2) : nullptr);
    }
    L.bytes = b.off + 256;
    return L;
}

int dfields(const vsz_dbatch_field* fields, int nfields, std::vector<DField>& out) {
    if (!fields || nfields <= 0) return VSZ_ERR_INVALID;
    out.clear();
    for (int i = 0; i < nfields; i++) {
        DField f{};
        VSZ_TRY(field_of(fields[i], f));
        // the kernel class: output rows of 16 bytes when the field's width and buffers allow
        DqDecArgs a{};
        a.d0         = f.g.d0;
        a.codes      = reinterpret_cast<const uint16_t*>(256);  // workspace codes are 256-byte aligned
        a.out        = fields[i].d_out;
        a.n          = f.g.n;
        a.n_outliers = fields[i].desc.n_outlier;
        a.redo       = reinterpret_cast<uint32_t*>(1);
        f.vec        = dq_b8_vec(a);
        f.sep        = dq_b8_separable(a, f.g.ndim);
        if (!f.sep) {  // the reference-order kernel groups narrow rows: its own unit count
            DqDecArgs t{};
            t.d0 = f.g.d0;
            t.d1 = f.g.d1;
            t.d2 = f.g.d2;
            dq_b8_geometry(t, f.g.ndim);
            dq_b8_narrow(t, f.g.ndim);
            f.units = t.nunits;
        }
        out.push_back(f);
    }
    return VSZ_OK;
}

}  // namespace

struct vsz_dbatch {
    int device = -1;
    int nfields = 0;
    uint8_t* d_tables = nullptr;  // owned: argument tables and task lists
    const ConstsField* consts = nullptr;
    const HuffTableArgs* table = nullptr;
    const HuffDecodeArgs* dec = nullptr;
    const DqDecArgs* dq = nullptr;
    const DCopy* copy_index = nullptr;
    const DCopy* copy_out = nullptr;
    const DCheck* check = nullptr;
    const BatchTask* tasks = nullptr;
    uint32_t idx_off = 0, idx_n = 0, dec_off = 0, dec_n = 0, const_off = 0, const_n = 0, out_off = 0, out_n = 0;
    uint32_t redo_off = 0, redo_n = 0;
    std::vector<DqClass> classes;
    uint8_t* ctl = nullptr;
    size_t ctl_bytes = 0;
    uint16_t* all_bits = nullptr;
    unsigned long long *all_start = nullptr, *all_zoff = nullptr;
    uint32_t* all_zero = nullptr;
    size_t total_chunks = 0;
    unsigned long long* scan_status = nullptr;
    uint32_t* scan_counter = nullptr;
    int* batch_status = nullptr;
};

extern "C" {

vsz_status vsz_dbatch_workspace_bytes(const vsz_dbatch_field* fields, int nfields, size_t* ws_bytes) {
    std::vector<DField> fs;
    VSZ_TRY(dfields(fields, nfields, fs));
    if (ws_bytes) *ws_bytes = layout_dbatch(fs, fields, nullptr, 0).bytes;
    return VSZ_OK;
}

vsz_status vsz_dbatch_create(const vsz_dbatch_field* fields, int nfields, void* d_ws, size_t ws_bytes, int* d_status,
                             vsz_dbatch** out) {
    if (!out || !d_ws || !d_status) return VSZ_ERR_INVALID;
    *out = nullptr;
    std::vector<DField> fs;
    VSZ_TRY(dfields(fields, nfields, fs));
    DLayout L = layout_dbatch(fs, fields, reinterpret_cast<uint8_t*>(d_ws), ws_bytes);
    if (L.bytes > ws_bytes) return VSZ_ERR_CAPACITY;
    const uint32_t nf = (uint32_t)nfields;
    std::vector<ConstsField> cs(nf);
    std::vector<HuffTableArgs> ta(nf);
    std::vector<HuffDecodeArgs> da(nf);
    std::vector<DqDecArgs> qa(nf);
    std::vector<DCopy> ci(nf), co(nf);
    std::vector<DCheck> ck(nf);
    std::vector<BatchTask> tasks;
    vsz_dbatch* B = new vsz_dbatch();
    B->nfields    = nfields;
    cudaGetDevice(&B->device);
    for (uint32_t f = 0; f < nf; f++) {
        const vsz_dbatch_field& F = fields[f];
        const vsz_archive_desc& d = F.desc;
        const DField& G           = fs[f];
        uint8_t* ctl              = L.ctl + (size_t)f * kDCtlBytes;
        Consts* consts            = reinterpret_cast<Consts*>(ctl + kDCtlConsts);
        int* status               = reinterpret_cast<int*>(ctl + kDCtlStatus);
        uint32_t* info            = reinterpret_cast<uint32_t*>(ctl + kDCtlInfo);
        const size_t base         = L.chunk_base[f];
        cs[f] = ConstsField{VSZ_MODE_ABS, G.ebf, nullptr, nullptr, consts, status};

        HuffTableArgs& t = ta[f];
        t                = HuffTableArgs{};
        t.huff           = F.d_archive + d.huff_offset;
        t.huff_bytes     = d.huff_bytes;
        t.dict           = G.nsym;
        t.max_nodes      = (uint32_t)(2 * G.nsym - 1);
        t.table          = L.table[f];
        t.child          = L.child[f];
        t.node_sym       = L.node_sym[f];
        t.parent         = L.parent[f];
        t.walk           = L.walk[f];
        t.table2         = L.table2[f];
        t.info           = info;
        t.status         = status;

        HuffDecodeArgs& h = da[f];
        h                 = HuffDecodeArgs{};
        h.payload         = F.d_archive + d.payload_offset;
        h.payload_bits    = (unsigned long long)d.payload_bytes * 8ull;
        h.table           = t.table;
        h.table2          = t.table2;
        h.child           = t.child;
        h.node_sym        = t.node_sym;
        h.walk            = t.walk;
        h.nodes           = d.node_count;
        h.start_bit       = L.all_start + base;
        h.chunk_len       = L.all_bits + base;
        h.chunk_zero      = L.all_zero + base;
        h.nchunks         = G.nch;
        h.chunk_syms      = kChunkSyms;
        h.codes           = L.code[f];
        h.n               = G.g.n;
        h.d0              = G.g.d0;
        h.nxs             = (G.g.d0 + 255) / 256;
        h.max_nodes       = (uint32_t)(2 * G.nsym - 1);
        h.tree_info       = info;
        h.status          = status;

        DqDecArgs& q  = qa[f];
        q             = DqDecArgs{};
        q.codes       = L.code[f];
        q.outliers    = L.outliers[f];
        q.n_outliers  = d.n_outlier;
        q.status      = status;
        q.chunk_off   = L.all_zoff + base;
        q.consts      = consts;
        q.out         = F.d_out;
        q.d0          = G.g.d0;
        q.d1          = G.g.d1;
        q.d2          = G.g.d2;
        q.n           = G.g.n;
        q.R           = d.dict_size / 2;
        q.xtail       = (G.g.ndim == 3 && (G.g.d0 % 8) != 0) ? (G.g.d0 & ~7u) : G.g.d0;
        q.redo        = L.redo[f];
        dq_b8_geometry(q, G.g.ndim);
        if (!G.sep) dq_b8_narrow(q, G.g.ndim);

        ci[f] = DCopy{F.d_archive + d.index_offset, reinterpret_cast<uint8_t*>(L.all_bits + base), status};
        co[f] = DCopy{F.d_archive + d.outlier_offset, reinterpret_cast<uint8_t*>(L.outliers[f]), status};
        ck[f] = DCheck{L.all_zoff + base, G.nch, d.n_outlier, consts, status, d_status + f, L.redo[f]};
    }
    // ---- task lists
    B->idx_off = (uint32_t)tasks.size();
    for (uint32_t f = 0; f < nf; f++) add_tasks(tasks, f, 2 * fs[f].nch, kCopyTaskBytes);
    B->idx_n   = (uint32_t)tasks.size() - B->idx_off;
    B->dec_off = (uint32_t)tasks.size();
    for (uint32_t f = 0; f < nf; f++)
        if (!fs[f].konst) add_tasks(tasks, f, fs[f].nch, kDecTaskChunks);
    B->dec_n     = (uint32_t)tasks.size() - B->dec_off;
    B->const_off = (uint32_t)tasks.size();
    for (uint32_t f = 0; f < nf; f++)
        if (fs[f].konst) add_tasks(tasks, f, fs[f].nch, kDecTaskChunks);
    B->const_n = (uint32_t)tasks.size() - B->const_off;
    B->out_off = (uint32_t)tasks.size();
    for (uint32_t f = 0; f < nf; f++) add_tasks(tasks, f, 4 * fields[f].desc.n_outlier, kCopyTaskBytes);
    B->out_n = (uint32_t)tasks.size() - B->out_off;
    std::map<std::tuple<int, bool, bool>, std::vector<uint32_t>> classes;
    for (uint32_t f = 0; f < nf; f++) classes[std::make_tuple(fs[f].g.ndim, fs[f].vec, fs[f].sep)].push_back(f);
    static_assert(kDqNextOff + 4 * kDqMaxClasses <= 256, "the counters fit the control tail");
    if (classes.size() > kDqMaxClasses) {  // 3 dimensionalities x aligned or not x separable or not
        delete B;
        return VSZ_ERR_INVALID;
    }
    for (auto& kv : classes) {
        DqClass c{};
        std::tie(c.ndim, c.vec, c.sep) = kv.first;
        c.task_off = (uint32_t)tasks.size();
        for (uint32_t f : kv.second) add_tasks(tasks, f, fs[f].units, kDqTaskUnits);
        c.ntasks = (uint32_t)tasks.size() - c.task_off;
        B->classes.push_back(c);
    }
    B->redo_off = (uint32_t)tasks.size();
    for (uint32_t f = 0; f < nf; f++)
        if (fs[f].sep) add_tasks(tasks, f, 1, 1);
    B->redo_n = (uint32_t)tasks.size() - B->redo_off;
    // ---- upload
    size_t off = 0;
    auto place = [&](size_t bytes) {
        off       = (off + 255) & ~(size_t)255;
        size_t at = off;
        off += bytes;
        return at;
    };
    const size_t o_cs = place(sizeof(ConstsField) * nf), o_ta = place(sizeof(HuffTableArgs) * nf),
                 o_da = place(sizeof(HuffDecodeArgs) * nf), o_qa = place(sizeof(DqDecArgs) * nf),
                 o_ci = place(sizeof(DCopy) * nf), o_co = place(sizeof(DCopy) * nf), o_ck = place(sizeof(DCheck) * nf),
                 o_tk = place(sizeof(BatchTask) * std::max<size_t>(tasks.size(), 1));
    const size_t table_bytes = off + 256;
    std::vector<uint8_t> h(table_bytes, 0);
    memcpy(h.data() + o_cs, cs.data(), sizeof(ConstsField) * nf);
    memcpy(h.data() + o_ta, ta.data(), sizeof(HuffTableArgs) * nf);
    memcpy(h.data() + o_da, da.data(), sizeof(HuffDecodeArgs) * nf);
    memcpy(h.data() + o_qa, qa.data(), sizeof(DqDecArgs) * nf);
    memcpy(h.data() + o_ci, ci.data(), sizeof(DCopy) * nf);
    memcpy(h.data() + o_co, co.data(), sizeof(DCopy) * nf);
    memcpy(h.data() + o_ck, ck.data(), sizeof(DCheck) * nf);
    if (!tasks.empty()) memcpy(h.data() + o_tk, tasks.data(), sizeof(BatchTask) * tasks.size());
    if (cudaMalloc(reinterpret_cast<void**>(&B->d_tables), table_bytes) != cudaSuccess) {
        delete B;
        return VSZ_ERR_NOMEM;
    }
    if (cudaMemcpy(B->d_tables, h.data(), table_bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
        vsz_dbatch_destroy(B);
        return VSZ_ERR_CUDA;
    }
    B->consts       = reinterpret_cast<const ConstsField*>(B->d_tables + o_cs);
    B->table        = reinterpret_cast<const HuffTableArgs*>(B->d_tables + o_ta);
    B->dec          = reinterpret_cast<const HuffDecodeArgs*>(B->d_tables + o_da);
    B->dq           = reinterpret_cast<const DqDecArgs*>(B->d_tables + o_qa);
    B->copy_index   = reinterpret_cast<const DCopy*>(B->d_tables + o_ci);
    B->copy_out     = reinterpret_cast<const DCopy*>(B->d_tables + o_co);
    B->check        = reinterpret_cast<const DCheck*>(B->d_tables + o_ck);
    B->tasks        = reinterpret_cast<const BatchTask*>(B->d_tables + o_tk);
    B->ctl          = L.ctl;
    B->ctl_bytes    = (size_t)nf * kDCtlBytes + 256;
    B->batch_status = L.batch_status;
    B->all_bits     = L.all_bits;
    B->all_start    = L.all_start;
    B->all_zero     = L.all_zero;
    B->all_zoff     = L.all_zoff;
    B->total_chunks = L.chunk_base.empty() ? 0 : L.chunk_base.back() + fs.back().nch;
    B->scan_status  = L.scan_status;
    B->scan_counter = L.scan_counter;
    *out            = B;
    return VSZ_OK;
}

vsz_status vsz_dbatch_decompress(vsz_dbatch* B, void* stream) {
    if (!B) return VSZ_ERR_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != B->device) return VSZ_ERR_INVALID;
    cudaStream_t st   = S(stream);
    const int sms     = num_sms();
    const uint32_t nf = (uint32_t)B->nfields;
    const uint32_t fb = (nf + 127) / 128;
    // control words (constants, status, tree info, the batch status) to zero, redo counts to zero
    VSZ_CUDA(cudaMemsetAsync(B->ctl, 0, B->ctl_bytes, st));
    k_dbatch_init<<<fb, 128, 0, st>>>(B->check, nf);
    count_launch();
    {
        StageTimer t(kStEbSetup, st);
        VSZ_TRY(launch_consts_batch(B->consts, nf, st));
    }
    {
        StageTimer t(kStDecTable, st);
        VSZ_TRY(launch_huff_table_batch(B->table, nf, st, sms));
    }
    {
        StageTimer t(kStDecScanIndex, st);
        if (B->idx_n) {
            k_dbatch_copy<<<std::min<uint32_t>(B->idx_n, (uint32_t)sms * 8), 256, 0, st>>>(B->copy_index,
                                                                                          B->tasks + B->idx_off, B->idx_n);
            count_launch();
        }
        VSZ_TRY(launch_scan_u16(B->all_bits, B->all_start, B->total_chunks, B->scan_status, B->scan_counter, nullptr,
                                B->batch_status, st));
    }
    {
        StageTimer t(kStHuffDecode, st);
        VSZ_TRY(launch_huff_decode_batch(B->dec, B->tasks + B->dec_off, B->dec_n, B->tasks + B->const_off,
                                         B->const_n, st, sms));
    }
    {
        StageTimer t(kStZeroScan, st);
        VSZ_TRY(launch_scan_u32(B->all_zero, B->all_zoff, B->total_chunks, B->scan_status, B->scan_counter,
                                B->all_zoff + B->total_chunks, B->batch_status, st));
        k_dbatch_check<<<fb, 128, 0, st>>>(B->check, nf, B->batch_status);
        count_launch();
    }
    if (B->out_n) {
        StageTimer t(kStOutlierCopy, st);
        k_dbatch_copy<<<std::min<uint32_t>(B->out_n, (uint32_t)sms * 8), 256, 0, st>>>(B->copy_out,
                                                                                      B->tasks + B->out_off, B->out_n);
        count_launch();
    }
    {
        StageTimer t(kStLorenzoDecompress, st);
        uint32_t* next = reinterpret_cast<uint32_t*>(B->ctl + B->nfields * kDCtlBytes + kDqNextOff);
        for (size_t i = 0; i < B->classes.size(); i++) {
            const DqClass& c = B->classes[i];
            VSZ_TRY(launch_dq_decompress_batch(B->dq, B->tasks + c.task_off, c.ntasks, c.ndim, c.vec, c.sep, next + i,
                                               st, sms));
        }
        VSZ_TRY(launch_dq_redo_batch(B->dq, B->tasks + B->redo_off, B->redo_n, st, sms));
    }
    k_dbatch_status<<<fb, 128, 0, st>>>(B->check, nf);
    count_launch();
    VSZ_CUDA(cudaGetLastError());
    return VSZ_OK;
}

void vsz_dbatch_destroy(vsz_dbatch* B) {
    if (!B) return;
    if (B->d_tables) cudaFree(B->d_tables);
    delete B;
}

}  // extern "C"
