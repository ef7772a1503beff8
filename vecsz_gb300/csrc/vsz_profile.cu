// Per-stage CUDA-event timing (see vsz_profile.h).  Event pairs are kept until vsz_profile_read,
// which synchronises on them and accumulates elapsed times.  Every stage is also an NVTX range
// (named as in vsz_profile_read), so a timeline tool shows the stages around their launches.
#include <atomic>
#include <cstdint>
#include <mutex>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "vsz_profile.h"
#include "vsz_types.h"

namespace vsz {

namespace {
std::mutex g_mu;
bool g_on = false;
struct Pair {
    int stage;
    cudaEvent_t a, b;
};
std::vector<Pair> g_pairs;
double g_ms[kStCount];
int g_cnt[kStCount];
const char* g_names[kStCount] = {"eb_setup",       "dualquant",   "huff_build",     "huff_count",
                                 "huff_pack",      "outlier_gather", "finalize",    "dec_table",
                                 "dec_index_scan", "huff_decode",  "zero_scan",      "outlier_copy",
                                 "lorenzo_decompress"};
}  // namespace

bool profile_on() { return g_on; }

namespace {
std::atomic<unsigned long long> g_launches{0};
}
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

StageTimer::StageTimer(int s, cudaStream_t stream) : stage(s), st(stream) {
    nvtxRangePushA(g_names[s]);
    if (!g_on) return;
    if (cudaEventCreate(&a) != cudaSuccess) {
        a = nullptr;
        return;
    }
    cudaEventRecord(a, st);
}

StageTimer::~StageTimer() {
    nvtxRangePop();
    if (!a) return;
    cudaEvent_t b;
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return;
    }
    cudaEventRecord(b, st);
    std::lock_guard<std::mutex> lk(g_mu);
    g_pairs.push_back(Pair{stage, a, b});
}

}  // namespace vsz

extern "C" {

void vsz_profile_enable(int on) { vsz::g_on = on != 0; }

uint64_t vsz_launch_count(void) { return vsz::g_launches.load(std::memory_order_relaxed); }

void vsz_profile_reset(void) {
    std::lock_guard<std::mutex> lk(vsz::g_mu);
    for (auto& p : vsz::g_pairs) {
        cudaEventSynchronize(p.b);
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    vsz::g_pairs.clear();
    for (int i = 0; i < vsz::kStCount; i++) {
        vsz::g_ms[i]  = 0;
        vsz::g_cnt[i] = 0;
    }
}

int vsz_profile_read(double* ms, int* counts, const char** names, int max_stages) {
    std::lock_guard<std::mutex> lk(vsz::g_mu);
    for (auto& p : vsz::g_pairs) {
        cudaEventSynchronize(p.b);
        float t = 0.f;
        if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) {
            vsz::g_ms[p.stage] += t;
            vsz::g_cnt[p.stage] += 1;
        }
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    vsz::g_pairs.clear();
    int n = vsz::kStCount < max_stages ? vsz::kStCount : max_stages;
    for (int i = 0; i < n; i++) {
        if (ms) ms[i] = vsz::g_ms[i];
        if (counts) counts[i] = vsz::g_cnt[i];
        if (names) names[i] = vsz::g_names[i];
    }
    return vsz::kStCount;
}

}  // extern "C"
