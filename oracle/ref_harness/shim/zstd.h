/* Declarations of the two zstd entry points the reference headers call
   (LosslessCompressor/ZSTD.hpp); the harness links the system libzstd. */
#pragma once
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
size_t ZSTD_compress(void* dst, size_t dstCapacity, const void* src, size_t srcSize, int compressionLevel);
size_t ZSTD_decompress(void* dst, size_t dstCapacity, const void* src, size_t compressedSize);
#ifdef __cplusplus
}
#endif
