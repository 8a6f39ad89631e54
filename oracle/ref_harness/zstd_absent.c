/* Linked into the reference harness on a host without libzstd: the two zstd
   entry points the reference's lossless stage calls (LosslessCompressor/ZSTD.hpp)
   return zstd's generic error code, so only that stage is unavailable there.
   The benchmark's CPU arm uses the NullLevelCompressor path and never calls
   them. */
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

size_t ZSTD_compress(void* dst, size_t dstCapacity, const void* src, size_t srcSize, int compressionLevel) {
    (void)dst; (void)dstCapacity; (void)src; (void)srcSize; (void)compressionLevel;
    return (size_t)-1;
}

size_t ZSTD_decompress(void* dst, size_t dstCapacity, const void* src, size_t compressedSize) {
    (void)dst; (void)dstCapacity; (void)src; (void)compressedSize;
    return (size_t)-1;
}

#ifdef __cplusplus
}
#endif
