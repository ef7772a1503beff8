// The chunking of the device gzip pass, shared by the encoder (deflate.cu), the decoder
// (inflate.cu) and the deflate index the host entry points write (vsz_host.cu): every chunk of the
// input is deflated on its own, its matches reach back no further than its own start.
#pragma once

namespace vsz {
constexpr int kDeflateChunk = 16384;  // input bytes per chunk (a zlib window holds it)
}  // namespace vsz
