// Host-side Huffman tree build (host_tree.cpp): the same tree, codebook and serialised bytes as
// k_huff_build, for the stream-ordered host-build step of vsz_compress.
#pragma once

#include <cstddef>
#include <cstdint>

namespace vsz {

// Bytes of the serialised tree after the 8-byte [BE nodeCount][BE dict] head.
size_t host_tree_bytes(uint32_t nc);

// hist[dict] -> cb_word/cb_len[dict] (right-aligned codeword, length; 0 = unused symbol),
// info[4] = {node count, tree bytes, max code length, node count}, head = [BE nc][BE hdr_dict][tree]
// (hdr_dict 0: dict).  Returns 0, or 1 when no symbol occurs (info is then all zero and head is
// not written).
int host_huffman_build(const uint64_t* hist, int dict, uint64_t* cb_word, uint8_t* cb_len, uint32_t* info,
                       uint8_t* head, int hdr_dict = 0);

}  // namespace vsz
