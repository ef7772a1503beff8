// Probe harness around the UNMODIFIED vecSZ reference, compiled from the reference's own
// sources by oracle/ref/Makefile into oracle/_ref/libvszref.so.
//
// TEST INFRASTRUCTURE ONLY.  It exists so that the C restatement in oracle/vsz_oracle.c and the
// golden fixtures under tests/golden/ can be pinned to what the reference itself computes.
// Nothing in the product links or loads it.  It builds only on x86-64 (the reference uses
// AVX intrinsics, src/dualquant.hh:6).
//
// Entry points drive the reference exactly the way its workflow does:
//   vszref_dualquant      -> per-block c_lorenzo_{1,2,3}d1l  (src/vecsz_interface.hh:108-140)
//   vszref_huffman_encode -> createHuffmanTree + encode_withTree (src/vecsz_interface.hh:160-161)
//   vszref_huffman_decode -> createHuffmanTree + decode_withTree (src/vecsz_interface.hh:307-308)
//   vszref_xlorenzo       -> per-block x_lorenzo_{1,2,3}d1l (src/vecsz_interface.hh:323-354)
//   vszref_compress       -> vecsz::interface::Compress<float,int> (src/vecsz_interface.hh:31)
//   vszref_compress_pad   -> the same with -p padding, on one OpenMP thread
//   vszref_decompress     -> vecsz::interface::Decompress<float,int> (src/vecsz_interface.hh:232)
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fcntl.h>
#include <omp.h>
#include <unistd.h>

#include "vecsz_interface.hh"

namespace {

// The reference logs every stage to stdout; silence it while it runs.
struct QuietStdout {
    int saved = -1;
    QuietStdout() {
        fflush(stdout);
        std::cout.flush();
        saved   = dup(1);
        int dn  = open("/dev/null", O_WRONLY);
        if (dn >= 0) { dup2(dn, 1); close(dn); }
    }
    ~QuietStdout() {
        fflush(stdout);
        std::cout.flush();
        if (saved >= 0) { dup2(saved, 1); close(saved); }
    }
};

ArgParse* make_args(int ndim, int d0, int d1, int d2, int bs, int dict, double eb, int r2r) {
    auto ap        = new ArgParse();
    ap->ndim       = ndim;
    ap->dim4       = {d0, d1, d2, 1};
    ap->block_size = bs;
    ap->dict_size  = dict;
    ap->radius     = dict / 2;
    ap->eb         = eb;
    ap->mode       = r2r ? "r2r" : "abs";
    ap->dtype      = "f32";
    return ap;
}

// The reference's 1D prequant writes up to one block past the end of the field and its 2D/3D
// edge prequant reads up to bs rows past it (the 2D/3D results never depend on those cells).
// Hand it a copy padded with zeros so those accesses stay inside memory we own.
float* padded_copy(const float* in, size_t n, size_t pad) {
    auto p = new float[n + pad]();
    memcpy(p, in, n * sizeof(float));
    return p;
}

size_t overrun_pad(int d0, int d1, int bs) { return (size_t)(bs + 2) * (size_t)d0 * (size_t)d1 + 2 * (size_t)bs + 64; }

}  // namespace

extern "C" {

// Prequant + Lorenzo for every block; dense int32 codes and dense outlier values (0 where
// code != 0), as the reference's Compress holds them before the gather.
int vszref_dualquant(const float* in, int ndim, int d0, int d1, int d2, int bs, int dict, double eb_final,
                     int32_t* code, float* outlier) {
    QuietStdout quiet;
    auto ap       = make_args(ndim, d0, d1, d2, bs, dict, eb_final, 0);
    auto dims_L16 = InitializeDims(ap);
    size_t len    = dims_L16[LEN];
    auto cfg      = new config_t(dict, eb_final);
    auto ebs_L4   = InitializeErrorBoundFamily(cfg);
    float* data   = padded_copy(in, len, overrun_pad(d0, d1, bs));
    memset(code, 0, len * sizeof(int32_t));
    memset(outlier, 0, len * sizeof(float));
    size_t pad_idx  = 0;
    float* pad_vals = nullptr;
    int vl          = MAX_VECTOR_LENGTH;
    if (ndim == 1) {
        for (size_t b0 = 0; b0 < dims_L16[nBLK0]; b0++)
            vecsz::predictor_quantizer::c_lorenzo_1d1l<float, int>(data, outlier, code, dims_L16, ebs_L4, b0, bs, vl,
                                                                  ap->szwf, ap->pad_constant, ap->pad_type, pad_vals,
                                                                  &pad_idx);
    } else if (ndim == 2) {
        for (size_t b1 = 0; b1 < dims_L16[nBLK1]; b1++)
            for (size_t b0 = 0; b0 < dims_L16[nBLK0]; b0++)
                vecsz::predictor_quantizer::c_lorenzo_2d1l<float, int>(data, outlier, code, dims_L16, ebs_L4, b0, b1,
                                                                      bs, vl, ap->szwf, ap->pad_constant, ap->pad_type,
                                                                      pad_vals, &pad_idx);
    } else {
        for (size_t b2 = 0; b2 < dims_L16[nBLK2]; b2++)
            for (size_t b1 = 0; b1 < dims_L16[nBLK1]; b1++)
                for (size_t b0 = 0; b0 < dims_L16[nBLK0]; b0++)
                    vecsz::predictor_quantizer::c_lorenzo_3d1l<float, int>(data, outlier, code, dims_L16, ebs_L4, b0,
                                                                          b1, b2, bs, vl, ap->szwf, ap->pad_constant,
                                                                          ap->pad_type, pad_vals, &pad_idx);
    }
    delete[] data;
    delete[] ebs_L4;
    delete cfg;
    delete[] dims_L16;
    delete ap;
    return 0;
}

// encode_withTree over int32 codes; *out is malloc'd (free with vszref_free).
int vszref_huffman_encode(const int32_t* code, size_t n, int dict, uint8_t** out, size_t* out_size) {
    QuietStdout quiet;
    auto tree = DesignVerification::createHuffmanTree(dict * 2);
    uint8_t* buf = nullptr;
    size_t sz    = 0;
    DesignVerification::encode_withTree(tree, code, n, &buf, &sz);
    *out      = (uint8_t*)malloc(sz ? sz : 1);
    memcpy(*out, buf, sz);
    *out_size = sz;
    free(buf);
    return 0;
}

// Codeword table the reference built for the last encode: lengths (cout) and the first 64-bit
// word of each codeword, for symbols [0, dict).
int vszref_huffman_codebook(const int32_t* code, size_t n, int dict, uint8_t* lens, uint64_t* words0,
                            uint64_t* words1) {
    QuietStdout quiet;
    auto tree = DesignVerification::createHuffmanTree(dict * 2);
    DesignVerification::initHuffman(tree, code, n);
    for (int i = 0; i < dict; i++) {
        lens[i]   = tree->cout[i];
        words0[i] = tree->code[i] ? tree->code[i][0] : 0;
        words1[i] = tree->code[i] ? tree->code[i][1] : 0;
    }
    return 0;
}

int vszref_huffman_decode(const uint8_t* huff, size_t n, int dict, int32_t* out) {
    QuietStdout quiet;
    auto tree = DesignVerification::createHuffmanTree(dict * 2);
    DesignVerification::decode_withTree(tree, huff, n, out);
    return 0;
}

// Reverse prediction-quantization from dense codes and dense outlier values.
int vszref_xlorenzo(const int32_t* code_in, const float* outlier_in, int ndim, int d0, int d1, int d2, int bs, int dict,
                    double eb_final, float* xdata) {
    QuietStdout quiet;
    auto ap       = make_args(ndim, d0, d1, d2, bs, dict, eb_final, 0);
    auto dims_L16 = InitializeDims(ap);
    size_t len    = dims_L16[LEN];
    auto cfg      = new config_t(dict, eb_final);
    auto ebs_L4   = InitializeErrorBoundFamily(cfg);
    auto code     = new int32_t[len];
    auto outlier  = new float[len];
    memcpy(code, code_in, len * sizeof(int32_t));
    memcpy(outlier, outlier_in, len * sizeof(float));
    size_t pad_idx = 0;
    float zero_pad[1] = {0.0f};  // the reference reads pad_vals[0] from an empty array here; use 0
    if (ndim == 1) {
        for (size_t b0 = 0; b0 < dims_L16[nBLK0]; b0++)
            vecsz::predictor_quantizer::x_lorenzo_1d1l<float, int>(xdata, outlier, code, dims_L16, ebs_L4[EBx2], b0, bs,
                                                                  ap->szwf, &pad_idx, zero_pad);
    } else if (ndim == 2) {
        for (size_t b1 = 0; b1 < dims_L16[nBLK1]; b1++)
            for (size_t b0 = 0; b0 < dims_L16[nBLK0]; b0++)
                vecsz::predictor_quantizer::x_lorenzo_2d1l<float, int>(xdata, outlier, code, dims_L16, ebs_L4[EBx2],
                                                                      b0, b1, bs, ap->szwf, &pad_idx, zero_pad);
    } else {
        for (size_t b2 = 0; b2 < dims_L16[nBLK2]; b2++)
            for (size_t b1 = 0; b1 < dims_L16[nBLK1]; b1++)
                for (size_t b0 = 0; b0 < dims_L16[nBLK0]; b0++)
                    vecsz::predictor_quantizer::x_lorenzo_3d1l<float, int>(xdata, outlier, code, dims_L16,
                                                                          ebs_L4[EBx2], b0, b1, b2, bs, ap->szwf,
                                                                          &pad_idx, zero_pad);
    }
    delete[] code;
    delete[] outlier;
    delete[] ebs_L4;
    delete cfg;
    delete[] dims_L16;
    delete ap;
    return 0;
}

// Full Compress<float,int>.  `tmpfile_path` must name a writable scratch file: the reference
// re-reads the input from disk for r2r (src/types.cc:28).  lossless: 0 none, 1 zstd, 2 gzip.
// *out is malloc'd: the packed block (lossless == 0) or the lossless frame.
int vszref_compress(const float* in, int ndim, int d0, int d1, int d2, int bs, int dict, double eb, int r2r,
                    int lossless, const char* tmpfile_path, uint8_t** out, size_t* data_size, size_t* lossless_size,
                    size_t* n_outlier) {
    auto ap               = make_args(ndim, d0, d1, d2, bs, dict, eb, r2r);
    size_t len            = (size_t)d0 * d1 * d2;
    ap->files.input_file  = tmpfile_path;
    if (lossless) {
        ap->szwf.lossless_pass = true;
        if (lossless == 2) ap->szwf.lossless_gzip = true;
        else ap->szwf.lossless_zstd = true;
    }
    FILE* f = fopen(tmpfile_path, "wb");
    if (!f) return 1;
    fwrite(in, sizeof(float), len, f);
    fclose(f);
    float* data            = padded_copy(in, len, overrun_pad(d0, d1, bs));
    size_t nout            = 0, dsz = 0;
    unsigned long lsz      = 0;
    unsigned char* res;
    {
        QuietStdout quiet;
        res = (unsigned char*)vecsz::interface::Compress<float, int>(ap, data, &nout, &dsz, &lsz);
    }
    size_t bytes = lossless ? lsz : dsz;
    *out         = (uint8_t*)malloc(bytes ? bytes : 1);
    memcpy(*out, res, bytes);
    if (lossless) free(res);
    else delete[] res;  // Compress already deleted `data` on this path (src/vecsz_interface.hh:222)
    if (lossless) delete[] data;
    *data_size     = dsz;
    *lossless_size = lsz;
    *n_outlier     = nout;
    delete ap;
    return 0;
}

// Compress<float,int> with padding (-p): pad_mode 1 global, 2 block, 3 edge; pad_type as
// src/utils/padding.hh:9-12.  Run on one OpenMP thread: the reference's blocks share one pad index
// (src/dualquant.hh:41), so with more threads the pad order, and the archive, vary run to run.
int vszref_compress_pad(const float* in, int ndim, int d0, int d1, int d2, int bs, int dict, double eb, int r2r,
                        int pad_mode, int pad_type, float pad_constant, const char* tmpfile_path, uint8_t** out,
                        size_t* data_size, size_t* n_outlier) {
    auto ap               = make_args(ndim, d0, d1, d2, bs, dict, eb, r2r);
    size_t len            = (size_t)d0 * d1 * d2;
    ap->files.input_file  = tmpfile_path;
    ap->szwf.global_padding = pad_mode == 1;
    ap->szwf.block_padding  = pad_mode == 2;
    ap->szwf.edge_padding   = pad_mode == 3;
    ap->pad_type            = pad_type;
    ap->pad_constant        = pad_constant;
    FILE* f = fopen(tmpfile_path, "wb");
    if (!f) return 1;
    fwrite(in, sizeof(float), len, f);
    fclose(f);
    float* data       = padded_copy(in, len, overrun_pad(d0, d1, bs));
    size_t nout       = 0, dsz = 0;
    unsigned long lsz = 0;
    unsigned char* res;
    const int threads = omp_get_max_threads();
    omp_set_num_threads(1);
    {
        QuietStdout quiet;
        res = (unsigned char*)vecsz::interface::Compress<float, int>(ap, data, &nout, &dsz, &lsz);
    }
    omp_set_num_threads(threads);
    *out = (uint8_t*)malloc(dsz ? dsz : 1);
    memcpy(*out, res, dsz);
    delete[] res;  // Compress deleted `data`
    *data_size = dsz;
    *n_outlier = nout;
    delete ap;
    return 0;
}

// Full Decompress<float,int> of a packed block (or lossless frame).  For r2r the reference reads
// the ORIGINAL field from `orig_file` to recover the value range (src/vecsz_interface.hh:280-284),
// which only the dry-run workflow supplies correctly.
int vszref_decompress(const uint8_t* payload, size_t data_size, size_t lossless_size, int bs, int dict, int r2r,
                      const char* orig_file, float* xdata, size_t n) {
    auto ap              = new ArgParse();
    ap->block_size       = bs;
    ap->dict_size        = dict;
    ap->radius           = dict / 2;
    ap->mode             = r2r ? "r2r" : "abs";
    ap->files.input_file = orig_file ? orig_file : "";
    size_t bytes         = lossless_size ? lossless_size : data_size;
    auto buf             = new unsigned char[bytes + 16]();
    memcpy(buf, payload, bytes);
    float* res;
    // one OpenMP thread: with padding the blocks share one pad index (src/dualquant.hh:923)
    const int threads = omp_get_max_threads();
    omp_set_num_threads(1);
    {
        QuietStdout quiet;
        res = (float*)vecsz::interface::Decompress<float, int>(ap, buf, data_size, lossless_size);
    }
    omp_set_num_threads(threads);
    memcpy(xdata, res, n * sizeof(float));
    delete[] res;
    delete ap;
    return 0;
}

void vszref_free(void* p) { free(p); }

}  // extern "C"
