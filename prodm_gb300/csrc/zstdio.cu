// Host decompression of level files written by the reference's lossless
// stage: AdaptiveLevelCompressor (AdaptiveLevelCompressor.hpp:13-60) stores a
// compressed bitplane as ZSTD::compress writes it (ZSTD.hpp:11-21): the raw
// length as an 8-byte size_t, then one zstd frame. The device codec of this
// library is ZCB (lossless.cu); zstd frames only come in with level files a
// stock refactor wrote, and they are expanded here, on the host, before the
// raw planes go to the device. libzstd is opened at run time (libzstd.so.1),
// so the library has no link-time dependency on it.
#include <dlfcn.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace prodm {

namespace {

struct ZstdApi {
    size_t (*decompress)(void*, size_t, const void*, size_t) = nullptr;
    unsigned (*is_error)(size_t) = nullptr;
    const char* (*error_name)(size_t) = nullptr;
};

const ZstdApi* zstd_api() {
    static ZstdApi api;
    static bool ok = false;
    static std::once_flag once;
    std::call_once(once, [] {
        void* h = nullptr;
        for (const char* name : {"libzstd.so.1", "libzstd.so"})
            if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
        if (!h) return;
        api.decompress = (size_t(*)(void*, size_t, const void*, size_t))dlsym(h, "ZSTD_decompress");
        api.is_error = (unsigned (*)(size_t))dlsym(h, "ZSTD_isError");
        api.error_name = (const char* (*)(size_t))dlsym(h, "ZSTD_getErrorName");
        ok = api.decompress && api.is_error && api.error_name;
    });
    return ok ? &api : nullptr;
}

}  // namespace

bool zstd_available() { return zstd_api() != nullptr; }

// One stored plane -> its raw bytes appended to out. A plane must hold the
// 8-byte raw length and a frame that expands to exactly that many bytes
// (ZSTD.hpp:22-28 reads the length the same way).
int zstd_expand_plane(const uint8_t* src, uint64_t stored, uint64_t max_raw, std::vector<uint8_t>& out) {
    const ZstdApi* z = zstd_api();
    if (!z)
        return fail(PRODM_EUNSUPPORTED, "level files compressed by the reference's zstd stage need libzstd.so.1, "
                                        "which could not be opened");
    if (stored < 8) return fail(PRODM_ECORRUPT, "zstd plane shorter than its raw-length header");
    uint64_t raw;
    std::memcpy(&raw, src, 8);
    if (raw > max_raw) return fail(PRODM_ECORRUPT, "zstd plane: raw length beyond the level's plane size");
    const size_t at = out.size();
    out.resize(at + raw);
    const size_t got = z->decompress(out.data() + at, (size_t)raw, src + 8, (size_t)(stored - 8));
    if (z->is_error(got)) {
        out.resize(at);
        return fail(PRODM_ECORRUPT, std::string("zstd plane: ") + z->error_name(got) +
                                        " (is the latter index the one the files were written with?)");
    }
    if (got != raw) {
        out.resize(at);
        return fail(PRODM_ECORRUPT, "zstd plane: frame size differs from its raw-length header");
    }
    return PRODM_OK;
}

}  // namespace prodm
