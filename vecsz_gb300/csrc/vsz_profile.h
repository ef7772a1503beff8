// Optional per-stage CUDA-event timing for the whole-field pipelines (vsz_profile_* in the C ABI).
#pragma once
#include <cuda_runtime.h>

namespace vsz {

enum Stage {
    kStEbSetup = 0,
    kStDualquant,
    kStHuffBuild,
    kStHuffCount,
    kStHuffPack,
    kStOutlierGather,
    kStFinalize,
    kStDecTable,
    kStDecScanIndex,
    kStHuffDecode,
    kStZeroScan,
    kStOutlierCopy,
    kStLorenzoDecompress,
    kStCount
};

bool profile_on();
// RAII pair of events around one stage on `st` (no-op when profiling is off).
struct StageTimer {
    int stage;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    StageTimer(int s, cudaStream_t stream);
    ~StageTimer();
};

}  // namespace vsz
