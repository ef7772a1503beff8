// Heap-tree Huffman codebook built on the host, for the stream-ordered host-build mode of
// vsz_compress (the library's tree thread answers k_tree_handoff between the histogram and the
// encoder).
//
// Same result as k_huff_build (huffman.cu): the reference's binary-heap priority queue replayed
// operation for operation (src/huffman.hh:169-192, 248-262; the first qremove() of a merge is the
// RIGHT child), preorder numbering of pad_tree_* (:374-423), codewords of build_code (:200-227),
// serialisation of convert_HuffTree_to_bytes_anyStates (:425-502).  The replay is a long chain of
// dependent, branchy memory operations on a few KB: one CPU core runs it several times faster than
// one GPU thread.
#include "host_tree.h"

#include <cstring>
#include <vector>

namespace vsz {

static inline uint32_t tree_width(uint32_t nc) { return nc <= 256 ? 1u : (nc <= 65536 ? 2u : 4u); }

size_t host_tree_bytes(uint32_t nc) {
    const size_t w = tree_width(nc);
    return 1 + 2 * w * nc + 4 * (size_t)nc + nc;
}

int host_huffman_build(const uint64_t* hist, int dict, uint64_t* cb_word, uint8_t* cb_len, uint32_t* info,
                       uint8_t* head, int hdr_dict) {
    std::vector<uint32_t> used;
    used.reserve((size_t)dict);
    for (int s = 0; s < dict; s++)
        if (hist[s]) used.push_back((uint32_t)s);
    const int nused = (int)used.size();
    std::memset(cb_word, 0, sizeof(uint64_t) * (size_t)dict);
    std::memset(cb_len, 0, (size_t)dict);
    info[0] = info[1] = info[2] = info[3] = 0u;
    if (nused == 0) return 1;  // the reference dereferences a null root here
    // children of internal nodes (creation order); the heap holds (freq, node) pairs so that its
    // comparisons read the entries themselves.  The operations and their order are the
    // reference's (qinsert huffman.hh:169, qremove :179), so ties resolve the same way.
    struct HeapEnt {
        uint64_t f;
        int32_t n;
    };
    std::vector<int32_t> lch((size_t)nused), rch((size_t)nused);
    // 1-based; qremove reads up to entry 4 i + 3 for a hole i with 2 i < qend <= nused + 1, so
    // 2 nused + 6 entries (value-initialised) cover every read
    std::vector<HeapEnt> heap(2 * (size_t)nused + 8);
    int qend = 1;
    auto qinsert = [&](uint64_t fn, int n) {
        int i = qend++, j;
        while ((j = i >> 1)) {
            if (heap[j].f <= fn) break;
            heap[i] = heap[j];
            i       = j;
        }
        heap[i] = HeapEnt{fn, n};
    };
    // The hole always sinks to the bottom (no early exit), moving up the smaller child, the left
    // one on a tie.  Two levels per pass: this level's choice and both possible choices of the
    // next level come from loads that do not wait on each other, and only the final select does.
    // No entry read is written in the same pass (the hole i is above its grandchildren 4 i ..
    // 4 i + 3), so each choice sees the values the one-level loop would see.  Reads at or past
    // qend are masked out of the choice.
    auto qremove = [&]() -> HeapEnt {
        const HeapEnt top = heap[1];
        qend--;
        int i = 1;
        for (;;) {
            const int l = i << 1;
            if (l >= qend) break;
            const int g   = l << 1;
            const bool p  = (l + 1 < qend) & (heap[l + 1].f < heap[l].f);
            const bool p0 = (g + 1 < qend) & (heap[g + 1].f < heap[g].f);
            const bool p1 = (g + 3 < qend) & (heap[g + 3].f < heap[g + 2].f);
            const int c   = l + (int)p;
            heap[i]       = heap[c];
            const int gc  = c << 1;  // g, or g + 2 when the right child moved up
            if (gc >= qend) {
                i = c;
                break;
            }
            const int cc = gc + (int)(p ? p1 : p0);
            heap[c]      = heap[cc];
            i            = cc;
        }
        heap[i] = heap[qend];
        return top;
    };
    for (int i = 0; i < nused; i++) qinsert(hist[used[i]], i);
    int nnodes = nused;
    while (qend > 2) {
        const HeapEnt r = qremove();
        const HeapEnt l = qremove();
        const int v     = nnodes++;
        lch[v - nused]  = l.n;
        rch[v - nused]  = r.n;
        qinsert(l.f + r.f, v);
    }
    // subtree sizes bottom-up, then preorder index / codeword / depth top-down
    const int nint = nnodes - nused;
    std::vector<uint32_t> size((size_t)nnodes, 1u), pre((size_t)nnodes, 0u), depth((size_t)nnodes, 0u);
    std::vector<uint64_t> code((size_t)nnodes, 0ull);
    for (int k = 0; k < nint; k++) size[nused + k] = 1u + size[lch[k]] + size[rch[k]];
    uint32_t max_len = 0;
    for (int k = nint - 1; k >= 0; k--) {
        const int v = nused + k, l = lch[k], r = rch[k];
        pre[l]   = pre[v] + 1u;
        pre[r]   = pre[v] + 1u + size[l];
        code[l]  = code[v] << 1;
        code[r]  = (code[v] << 1) | 1ull;
        depth[l] = depth[r] = depth[v] + 1u;
        if (depth[l] > max_len) max_len = depth[l];
    }
    const uint32_t nc = (uint32_t)nnodes;
    // [BE nodeCount][BE dict][u8 0][L][R][C u32 LE][t]
    const uint32_t w = tree_width(nc);
    head[0] = (uint8_t)(nc >> 24);
    head[1] = (uint8_t)(nc >> 16);
    head[2] = (uint8_t)(nc >> 8);
    head[3] = (uint8_t)nc;
    const uint32_t dh = (uint32_t)(hdr_dict ? hdr_dict : dict);
    head[4] = (uint8_t)(dh >> 24);
    head[5] = (uint8_t)(dh >> 16);
    head[6] = (uint8_t)(dh >> 8);
    head[7] = (uint8_t)dh;
    head[8] = 0;
    uint8_t* pL = head + 9;
    uint8_t* pR = pL + (size_t)w * nc;
    uint8_t* pC = pR + (size_t)w * nc;
    uint8_t* pT = pC + 4 * (size_t)nc;
    std::memset(pL, 0, 2 * (size_t)w * nc);
    for (int v = 0; v < nnodes; v++) {
        const uint32_t idx = pre[v];
        uint32_t c = 0, lv = 0, rv = 0;
        const bool leaf = v < nused;
        if (leaf) {
            c          = used[v];
            cb_len[c]  = (uint8_t)(depth[v] > 255u ? 255u : depth[v]);
            cb_word[c] = code[v];
        } else {
            lv = pre[lch[v - nused]];
            rv = pre[rch[v - nused]];
        }
        for (uint32_t b = 0; b < w; b++) {
            pL[(size_t)idx * w + b] = (uint8_t)(lv >> (8 * b));
            pR[(size_t)idx * w + b] = (uint8_t)(rv >> (8 * b));
        }
        std::memcpy(pC + 4 * (size_t)idx, &c, 4);
        pT[idx] = leaf ? 1 : 0;
    }
    info[0] = nc;
    info[1] = (uint32_t)host_tree_bytes(nc);
    info[2] = max_len;
    info[3] = nc;
    return 0;
}

}  // namespace vsz
