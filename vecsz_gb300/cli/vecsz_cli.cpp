// `vecsz`: the reference's command line (src/vecsz.cc main, src/argument_parser/argparse.cc) over
// this library's host entry points.  Same flags, defaults, output naming and .sz file layout
// ([u64 lossless_size][u64 data_size][payload]); compress (-z), decompress (-x) and dry-run (-r)
// run on the GPU.  Built by vecsz_gb300/_build.py into vecsz_gb300/_lib/vecsz.
#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "vecsz_gb300.h"

namespace {

struct Args {
    bool compress = false, decompress = false, dryrun = false;
    bool verbose = false, skip_write = false, show_histo = false, autotune = false;
    std::string mode = "abs", dtype, input, output, demo, padding, lossless;
    bool lossless_pass = false;
    double eb = 1e-4, sample_percentage = -1;
    int num_iterations = -1;
    int ndim = -1;
    long dims[4] = {1, 1, 1, 1};
    int dict_size = 4096, block_size = 8;
    bool bad = false;
};

void usage(bool full) {
    std::printf(
        "vecsz (GB300): SZ dual-quantization compression on the GPU\n\n"
        "  -z, --compress, --zip        compress the input file\n"
        "  -x, --decompress, --unzip    decompress a .sz file\n"
        "  -r, --dry-run                compress, decompress and report the error metrics\n"
        "  -t, --dtype f32|f64          data type (f64: the double-precision path, error bound guaranteed)\n"
        "  -m, --mode abs|r2r           error-bound mode (default abs)\n"
        "  -e, --eb <value>             error bound (default 1e-4)\n"
        "  -l, --len x[,y[,z]]          dimensions, fastest first\n"
        "  -D, --demo <name>            dimensions of a named dataset (nyx, cesm, hurricane, ...)\n"
        "  -i, --input <file>           input file\n"
        "  -o, --output <file>          output file (default <input>.sz, <input>.out, <input>.sz.out)\n"
        "  -d, --dict-size <n>          quantization dictionary size (default 4096)\n"
        "  -b, --block-size <n>         block size 8, 16, 32 or 64 (default 8)\n"
        "  -p, --padding <spec>         global|block|edge with max|min|avg|constant [value]\n"
        "  -L, --lossless gzip|zstd|gzip-gpu  lossless pass over the archive\n"
        "  -a, --autotune               choose the block size on the GPU (--num-iter, --sample)\n"
        "  -S, --skip write             do not write the output file\n"
        "  -s, --vector <len>           accepted for compatibility; the GPU path has no vector width\n"
        "  -V, --verbose                print the configuration and timings\n"
        "  -v, --version                print the version\n"
        "  -h, --help                   this text\n");
    if (full) std::printf("\nLibrary: %s\n", vsz_version());
}

long to_long(const std::string& s, bool* bad) {
    char* end = nullptr;
    errno     = 0;
    long v    = std::strtol(s.c_str(), &end, 10);
    if (s.empty() || *end || errno) {
        std::fprintf(stderr, "[error] invalid option value, non-convertible part: %s\n", s.c_str());
        *bad = true;
    }
    return v;
}

Args parse(int argc, char** argv) {
    Args a;
    if (argc == 1) {
        usage(false);
        std::exit(0);
    }
    auto next = [&](int& i) -> std::string {
        if (i + 1 < argc) return std::string(argv[++i]);
        std::fprintf(stderr, "[error] option %s needs a value\n", argv[i]);
        a.bad = true;
        return std::string();
    };
    for (int i = 1; i < argc; i++) {
        const std::string o = argv[i];
        if (o.size() < 2 || o[0] != '-') {
            std::fprintf(stderr, "[error] invalid option at position %d: %s\n", i, argv[i]);
            a.bad = true;
            continue;
        }
        const std::string L = o.size() > 2 && o[1] == '-' ? o : std::string();
        const char c        = L.empty() ? o[1] : 0;
        if (c == 'z' || L == "--compress" || L == "--zip") a.compress = true;
        else if (c == 'x' || L == "--decompress" || L == "--unzip") a.decompress = true;
        else if (c == 'r' || L == "--dry-run") a.dryrun = true;
        else if (c == 'm' || L == "--mode") a.mode = next(i);
        else if (c == 'e' || L == "--eb") a.eb = std::strtod(next(i).c_str(), nullptr);
        else if (c == 'd' || L == "--dict-size") a.dict_size = (int)to_long(next(i), &a.bad);
        else if (c == 'b' || L == "--block-size") a.block_size = (int)to_long(next(i), &a.bad);
        else if (c == 'i' || L == "--input") a.input = next(i);
        else if (c == 'o' || L == "--output") a.output = next(i);
        else if (c == 'D' || L == "--demo") a.demo = next(i);
        else if (c == 'p' || L == "--padding") a.padding = next(i);
        else if (c == 'V' || L == "--verbose") a.verbose = true;
        else if (c == 'a' || L == "--autotune") {
            a.autotune          = true;
            a.num_iterations    = 10;
            a.sample_percentage = 1.0;
        } else if (L == "--num-iter") a.num_iterations = (int)to_long(next(i), &a.bad);
        else if (L == "--sample") a.sample_percentage = std::strtod(next(i).c_str(), nullptr);
        else if (L == "--show-histo") a.show_histo = true;
        else if (c == 'h' || L == "--help") {
            usage(true);
            std::exit(0);
        } else if (c == 'v' || L == "--version") {
            std::printf("[info] %s\n", vsz_version());
            std::exit(0);
        } else if (c == 't' || L == "--dtype") {
            const std::string s = next(i);
            if (s == "f32" || s == "fp4") a.dtype = "f32";
            else if (s == "f64" || s == "fp8") a.dtype = "f64";
        } else if (c == 'L' || L == "--lossless") {
            a.lossless_pass = true;
            a.lossless      = next(i);
        } else if (c == 'S' || L == "--skip") {
            // the reference maps both "write" and "verify" to skipping the output file
            const std::string s = next(i);
            if (s.find("write") != std::string::npos || s.find("verify") != std::string::npos) a.skip_write = true;
            if (s.find("huffman") != std::string::npos)
                std::fprintf(stderr, "[warn] -S huffman: the Huffman stage always runs on the GPU path\n");
        } else if (c == 's' || L == "--vector") {
            (void)next(i);  // the AVX vector width of the reference's CPU path
        } else if (c == 'l' || L == "--len") {
            std::stringstream ss(next(i));
            std::string part;
            int k = 0;
            while (std::getline(ss, part, ',')) {
                if (k < 4) a.dims[k] = to_long(part, &a.bad);
                k++;
            }
            a.ndim = k;
            if (k < 1 || k > 4) {
                std::fprintf(stderr, "[error] Incorrect input size(s)!\n");
                a.bad = true;
            }
        } else {
            std::fprintf(stderr, "[error] invalid option value at position %d: %s\n", i, argv[i]);
            a.bad = true;
        }
    }
    if (a.bad) {
        std::printf("[info] Exiting...\n");
        std::exit(-1);
    }
    return a;
}

bool demo_dims(const std::string& name, Args& a) {
    // dataset entries of src/dimensions.hh:14-20: x, y, z, w, ndim
    static const std::map<std::string, std::vector<long>> table = {
        {"hacc", {280953867, 1, 1, 1, 1}}, {"hacc1b", {1073726487, 1, 1, 1, 1}}, {"cesm", {3600, 1800, 1, 1, 2}},
        {"hurricane", {500, 500, 100, 1, 3}}, {"nyx", {512, 512, 512, 1, 3}}, {"nyx-m", {1024, 1024, 1024, 1, 3}},
        {"qmc", {288, 69, 7935, 1, 3}}, {"qmcpre", {69, 69, 33120, 1, 3}}, {"exafel", {388, 59200, 1, 1, 2}},
        {"aramco", {235, 849, 849, 1, 3}}, {"parihaka", {1168, 1126, 922, 1, 3}}};
    auto it = table.find(name);
    if (it == table.end()) return false;
    for (int k = 0; k < 4; k++) a.dims[k] = it->second[k];
    a.ndim = (int)it->second[4];
    return true;
}

void check(Args& a) {
    bool abort = false;
    if (a.input.empty()) {
        std::fprintf(stderr, "[error] Not specifying input file!\n");
        abort = true;
    }
    if (!a.demo.empty() && !demo_dims(a.demo, a)) {
        std::fprintf(stderr, "[error] unknown demo dataset: %s\n", a.demo.c_str());
        abort = true;
    }
    if ((a.compress || a.dryrun) && a.ndim < 0) {
        std::fprintf(stderr, "[error] Incorrect input size(s)!\n");
        abort = true;
    }
    if (!a.compress && !a.decompress && !a.dryrun) {
        std::fprintf(stderr, "[error] Select compress (-z), decompress (-x), or dry-run (-r)!\n");
        abort = true;
    }
    if ((a.compress || a.dryrun) && a.dtype != "f32" && a.dtype != "f64") {
        std::fprintf(stderr, "[error] Not specifying data type!\n");
        abort = true;
    }
    if (a.dict_size > 65536) {
        std::fprintf(stderr, "[error] dictionary size above 65536\n");
        abort = true;
    }
    if (a.ndim == 4) {  // the path is at most 3D: a trailing 1 folds away
        if (a.dims[3] != 1) {
            std::fprintf(stderr, "[error] 4D fields are not supported (x, y, z, 1 is)\n");
            abort = true;
        }
        a.ndim = 3;
    }
    if (a.dryrun && (a.compress || a.decompress)) {
        std::fprintf(stderr, "[warn] No need to dry-run and compress or decompress at the same time!\n");
        std::fprintf(stderr, "[warn] Will dry-run only.\n");
        a.compress = a.decompress = false;
    }
    if (a.compress && a.decompress) {
        std::fprintf(stderr, "[warn] Compress and decompress at once: will compress only.\n");
        a.decompress = false;
    }
    if (!a.autotune && (a.num_iterations >= 0 || a.sample_percentage >= 0)) {
        std::fprintf(stderr,
                     "[error] Autotune option not specified! Specify `-a` or `--autotune` to use `--sample` or "
                     "`--num-iter` options.\n");
        abort = true;
    }
    if (a.autotune) {
        if (a.num_iterations <= 0) a.num_iterations = 10;
        if (a.sample_percentage <= 0) a.sample_percentage = 1.0;
    }
    if (a.lossless_pass && a.lossless != "gzip" && a.lossless != "GZIP" && a.lossless != "zstd" &&
        a.lossless != "ZSTD" && a.lossless != "gzip-gpu") {
        std::fprintf(stderr, "[warn] No lossless compressor detected for -L option, defaulting to Gzip.\n");
        a.lossless = "gzip";
    }
    if (a.output.empty()) {
        if (a.compress) a.output = a.input + ".sz";
        if (a.decompress) a.output = a.input + ".out";
        if (a.dryrun) a.output = a.input + ".sz.out";
    }
    if (abort) {
        usage(false);
        std::exit(-1);
    }
}

[[noreturn]] void fail(const char* what, int st) {
    std::fprintf(stderr, "[error] %s: %s\n", what, vsz_status_string(st));
    std::exit(-1);
}

std::vector<uint8_t> read_file(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        std::fprintf(stderr, "[error] cannot open %s\n", path.c_str());
        std::exit(-1);
    }
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::vector<uint8_t> b(n > 0 ? (size_t)n : 0);
    if (n > 0 && std::fread(b.data(), 1, b.size(), f) != b.size()) {
        std::fprintf(stderr, "[error] cannot read %s\n", path.c_str());
        std::exit(-1);
    }
    std::fclose(f);
    return b;
}

void write_file(const std::string& path, const std::vector<std::pair<const void*, size_t>>& parts) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) {
        std::fprintf(stderr, "[error] cannot write %s\n", path.c_str());
        std::exit(-1);
    }
    for (const auto& p : parts)
        if (p.second && std::fwrite(p.first, 1, p.second, f) != p.second) {
            std::fprintf(stderr, "[error] cannot write %s\n", path.c_str());
            std::exit(-1);
        }
    std::fclose(f);
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

vsz_params params_of(const Args& a) {
    vsz_params p = {};
    p.eb         = a.eb;
    p.mode       = a.mode == "r2r" ? VSZ_MODE_R2R : VSZ_MODE_ABS;
    p.dict_size  = a.dict_size;
    p.block_size = a.block_size;
    p.lossless   = !a.lossless_pass                ? VSZ_LOSSLESS_NONE
                   : a.lossless == "gzip-gpu"      ? VSZ_LOSSLESS_GZIP_DEVICE
                   : (a.lossless == "zstd" || a.lossless == "ZSTD") ? VSZ_LOSSLESS_ZSTD
                                                                    : VSZ_LOSSLESS_GZIP;
    p.pad_type = VSZ_PADV_CONST;
    if (!a.padding.empty()) {
        const int st = vsz_parse_padding(a.padding.c_str(), &p);
        if (st != VSZ_OK) fail("padding", st);
    }
    return p;
}

// error metrics of a reconstruction (max absolute error and its index, value range, PSNR,
// NRMSE, correlation), as the reference's dry run prints them
template <typename T>
void print_metrics(const T* o, const T* x, size_t n, size_t archive_bytes) {
    double mn = o[0], mx = o[0], s0 = 0, sx = 0;
    for (size_t i = 0; i < n; i++) {
        mn = std::min(mn, (double)o[i]);
        mx = std::max(mx, (double)o[i]);
        s0 += o[i];
        sx += x[i];
    }
    const double m0 = s0 / n, mxm = sx / n;
    double maxerr = 0, maxrel = 0, sse = 0, cov = 0, v0 = 0, vx = 0;
    size_t imax = 0;
    for (size_t i = 0; i < n; i++) {
        const double e = std::fabs((double)x[i] - (double)o[i]);
        if (e > maxerr) maxerr = e, imax = i;
        if (o[i] != 0) maxrel = std::max(maxrel, e / std::fabs((double)o[i]));
        sse += e * e;
        cov += (o[i] - m0) * (x[i] - mxm);
        v0 += (o[i] - m0) * (o[i] - m0);
        vx += (x[i] - mxm) * (x[i] - mxm);
    }
    const double range = mx - mn, mse = sse / n;
    std::printf("\n");
    std::printf("  %-20s%.20G\n", "min.val", mn);
    std::printf("  %-20s%.20G\n", "max.val", mx);
    std::printf("  %-20s%.20G\n", "val.rng", range);
    std::printf("  %-20s%.20G\n", "max.err.abs.val", maxerr);
    std::printf("  %-20s%zu\n", "data.length", n);
    std::printf("  %-20s%zu\n", "max.err.abs.idx", imax);
    std::printf("  %-20s%.20G\n", "max.err.vs.rng", range > 0 ? maxerr / range : 0.0);
    std::printf("  %-20s%.20G\n", "max.pw.rel.err", maxrel);
    std::printf("  %-20s%.20G\n", "PSNR", 20 * std::log10(range) - 10 * std::log10(mse));
    std::printf("  %-20s%.20G\n", "NRMSE", std::sqrt(mse) / range);
    std::printf("  %-20s%.20G\n", "correl.coeff", cov / std::sqrt(v0 * vx));
    if (archive_bytes) std::printf("  %-20s%lf\n", "comp.ratio.w/o.gzip", 4.0 * n / archive_bytes);
    std::printf("\n");
}

template <typename T>
void print_histogram(const char* title, const T* v, size_t n, int bins) {
    double mn = v[0], mx = v[0];
    for (size_t i = 0; i < n; i++) mn = std::min(mn, (double)v[i]), mx = std::max(mx, (double)v[i]);
    std::vector<size_t> h(bins, 0);
    const double w = (mx - mn) / bins;
    for (size_t i = 0; i < n; i++) {
        int b = w > 0 ? (int)((v[i] - mn) / w) : 0;
        h[std::min(b, bins - 1)]++;
    }
    size_t peak = 1;
    for (size_t c : h) peak = std::max(peak, c);
    std::printf("\n  histogram of %s\n", title);
    for (int b = 0; b < bins; b++)
        std::printf("  %14.6g | %-50s %zu\n", mn + b * w, std::string((size_t)(50.0 * h[b] / peak), '#').c_str(),
                    h[b]);
}

size_t element_count(const Args& a) {
    size_t n = 1;
    for (int k = 0; k < a.ndim; k++) n *= (size_t)a.dims[k];
    return n;
}

template <typename T = float>
std::vector<T> read_field(const Args& a, size_t n) {
    std::vector<uint8_t> raw = read_file(a.input);
    if (raw.size() < sizeof(T) * n) {
        std::fprintf(stderr, "[error] %s holds %zu bytes, the dimensions need %zu\n", a.input.c_str(), raw.size(),
                     sizeof(T) * n);
        std::exit(-1);
    }
    std::vector<T> x(n);
    std::memcpy(x.data(), raw.data(), sizeof(T) * n);
    return x;
}

// -t f64: the f64 path (error bound guaranteed, 8-byte outliers); the reference reads f32 here
std::vector<uint8_t> compress_f64(const Args& a, vsz_params& p, const double* x, size_t* data_size,
                                  size_t* lossless_size) {
    const size_t dims[3] = {(size_t)a.dims[0], (size_t)a.dims[1], (size_t)a.dims[2]};
    if (a.autotune) std::fprintf(stderr, "[warn] -a: the block-size autotuner takes f32 fields; -b %d kept\n", p.block_size);
    uint8_t* out = nullptr;
    size_t ob = 0, no = 0;
    const auto t0 = std::chrono::steady_clock::now();
    const int st  = vsz_compress_host_f64(&p, a.ndim, dims, x, &out, &ob, data_size, lossless_size, &no);
    if (st != VSZ_OK) fail("compress", st);
    std::vector<uint8_t> payload(out, out + ob);
    vsz_free_host(out);
    if (a.verbose)
        std::printf("[dbg] compress (f64): %zu outliers, packed block %zu bytes, lossless %zu bytes, %.6f s\n", no,
                    *data_size, *lossless_size, seconds_since(t0));
    return payload;
}

std::vector<double> decompress_f64(const Args& a, const uint8_t* payload, size_t len, size_t data_size,
                                   size_t lossless_size) {
    double* out   = nullptr;
    size_t n      = 0;
    const int st  = vsz_decompress_host_f64(payload, len, data_size, lossless_size, &out, &n);
    if (st != VSZ_OK) fail("decompress", st);
    std::vector<double> y(out, out + n);
    vsz_free_host(out);
    if (a.verbose) std::printf("[dbg] decompress (f64): %zu values\n", n);
    return y;
}

// compress: returns the payload main() writes after its 16-byte header
std::vector<uint8_t> compress(const Args& a, vsz_params& p, const float* x, size_t* data_size,
                              size_t* lossless_size) {
    const size_t dims[3] = {(size_t)a.dims[0], (size_t)a.dims[1], (size_t)a.dims[2]};
    if (a.autotune) {
        int best = p.block_size;
        double ms[4];
        const int st =
            vsz_autotune_block_size_host(&p, a.ndim, dims, x, a.sample_percentage, a.num_iterations, &best, ms);
        if (st != VSZ_OK) fail("autotune", st);
        if (a.verbose)
            std::printf("[dbg] autotune: block size %d (8: %.4f ms, 16: %.4f ms, 32: %.4f ms, 64: %.4f ms)\n", best,
                        ms[0], ms[1], ms[2], ms[3]);
        p.block_size = best;
    }
    uint8_t* out = nullptr;
    size_t ob = 0, no = 0;
    const auto t0 = std::chrono::steady_clock::now();
    const int st  = vsz_compress_host(&p, a.ndim, dims, x, &out, &ob, data_size, lossless_size, &no);
    if (st != VSZ_OK) fail("compress", st);
    const double dt = seconds_since(t0);
    std::vector<uint8_t> payload(out, out + ob);
    vsz_free_host(out);
    if (a.verbose)
        std::printf("[dbg] compress: %zu outliers, packed block %zu bytes, lossless %zu bytes, %.6f s\n", no,
                    *data_size, *lossless_size, dt);
    return payload;
}

std::vector<float> decompress(const Args& a, const uint8_t* payload, size_t len, size_t data_size,
                              size_t lossless_size) {
    vsz_decompress_opts o = {};
    o.dict_size           = a.dict_size;
    o.block_size          = a.block_size;
    o.mode                = a.mode == "r2r" ? VSZ_MODE_R2R : VSZ_MODE_ABS;
    o.value_range         = 0;
    float* out            = nullptr;
    size_t n              = 0;
    const auto t0         = std::chrono::steady_clock::now();
    const int st          = vsz_decompress_host(payload, len, data_size, lossless_size, &o, &out, &n);
    if (st == VSZ_ERR_UNSUPPORTED) return {};  // an f64 archive: the caller takes decompress_f64
    if (st != VSZ_OK) fail("decompress", st);
    if (a.verbose) std::printf("[dbg] decompress: %zu values, %.6f s\n", n, seconds_since(t0));
    std::vector<float> y(out, out + n);
    vsz_free_host(out);
    return y;
}

}  // namespace

int main(int argc, char** argv) {
    Args a = parse(argc, argv);
    check(a);
    if (a.verbose) {
        std::printf("[cfg] Workflow:            %s\n", a.compress ? "compress" : a.decompress ? "decompress" : "dry-run");
        std::printf("[cfg] Input / output:      %s -> %s%s\n", a.input.c_str(), a.output.c_str(),
                    a.skip_write ? " (not written)" : "");
        std::printf("[cfg] Error mode / bound:  %s %g\n", a.mode.c_str(), a.eb);
        std::printf("[cfg] Dimensions (x,y,z):  (%ld,%ld,%ld), %d-D\n", a.dims[0], a.dims[1], a.dims[2], a.ndim);
        std::printf("[cfg] Dict. size / block:  %d / %d\n", a.dict_size, a.block_size);
        std::printf("[cfg] Lossless pass:       %s\n", a.lossless_pass ? a.lossless.c_str() : "no");
        std::printf("[cfg] Library:             %s\n", vsz_version());
    }
    if (a.dtype == "f64" && (a.compress || a.dryrun)) {
        const size_t n        = element_count(a);
        std::vector<double> x = read_field<double>(a, n);
        vsz_params p          = params_of(a);
        size_t ds = 0, ls = 0;
        std::vector<uint8_t> payload = compress_f64(a, p, x.data(), &ds, &ls);
        if (a.compress) {
            if (!a.skip_write) {
                const uint64_t head[2] = {(uint64_t)ls, (uint64_t)ds};
                write_file(a.output, {{head, sizeof(head)}, {payload.data(), payload.size()}});
            }
            return 0;
        }
        std::vector<double> y = decompress_f64(a, payload.data(), payload.size(), ds, ls);
        if (!a.skip_write) write_file(a.output, {{y.data(), 8 * y.size()}});
        if (a.show_histo) {
            print_histogram("original datum", x.data(), n, 16);
            print_histogram("reconstructed data", y.data(), n, 16);
        }
        print_metrics(x.data(), y.data(), n, ds);
        return 0;
    }

    if (a.compress) {
        const size_t n       = element_count(a);
        std::vector<float> x = read_field(a, n);
        vsz_params p         = params_of(a);
        size_t ds = 0, ls = 0;
        std::vector<uint8_t> payload = compress(a, p, x.data(), &ds, &ls);
        if (!a.skip_write) {
            const uint64_t head[2] = {(uint64_t)ls, (uint64_t)ds};
            write_file(a.output, {{head, sizeof(head)}, {payload.data(), payload.size()}});
            if (a.verbose) std::printf("[info] write %s %zu bytes\n", a.output.c_str(), payload.size() + 16);
        }
        return 0;
    }
    if (a.decompress) {
        std::vector<uint8_t> f = read_file(a.input);
        if (f.size() < 16) {
            std::fprintf(stderr, "[error] %s is not a .sz file\n", a.input.c_str());
            return -1;
        }
        uint64_t head[2];
        std::memcpy(head, f.data(), 16);
        std::vector<float> y = decompress(a, f.data() + 16, f.size() - 16, head[1], head[0]);
        if (y.empty()) {  // an f64 archive (its trailer says so): doubles out
            std::vector<double> z = decompress_f64(a, f.data() + 16, f.size() - 16, head[1], head[0]);
            if (!a.skip_write) write_file(a.output, {{z.data(), 8 * z.size()}});
            return 0;
        }
        if (!a.skip_write) write_file(a.output, {{y.data(), 4 * y.size()}});
        return 0;
    }
    // dry run
    const size_t n       = element_count(a);
    std::vector<float> x = read_field(a, n);
    vsz_params p         = params_of(a);
    size_t ds = 0, ls = 0;
    std::vector<uint8_t> payload = compress(a, p, x.data(), &ds, &ls);
    std::vector<float> y         = decompress(a, payload.data(), payload.size(), ds, ls);
    if (y.size() != n) {
        std::fprintf(stderr, "[error] decompressed %zu values, expected %zu\n", y.size(), n);
        return -1;
    }
    if (!a.skip_write) write_file(a.output, {{y.data(), 4 * y.size()}});
    if (a.show_histo) {
        print_histogram("original datum", x.data(), n, 16);
        print_histogram("reconstructed data", y.data(), n, 16);
    }
    print_metrics(x.data(), y.data(), n, ds);
    return 0;
}
