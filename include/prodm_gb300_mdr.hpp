// prodm_gb300 C++ plugin adapters -- header only, over the C ABI in
// prodm_gb300.h.
//
// Each class implements one of ProDM's MDR plugin concepts with exactly the
// reference's method signatures, so it can be passed as a template argument
// to MDR::ComposedRefactor / MDR::ComposedReconstructor
// (ComposedRefactor.hpp:15-16, ComposedReconstructor.hpp:17-18), which compose
// by template parameter:
//
//   DecomposerInterface<T>        (DecomposerInterface.hpp:14-16)   -> GpuMGARDDecomposer
//   InterleaverInterface<T>       (InterleaverInterface.hpp:14-16)  -> GpuDirectInterleaver
//   BitplaneEncoderInterface<T>   (BitplaneEncoderInterface.hpp:16-20)
//                                                        -> GpuNegaBinaryBPEncoder / GpuGroupedBPEncoder
//   ErrorCollectorInterface<T>    (ErrorCollectorInterface.hpp:14)  -> GpuMaxErrorCollector / GpuSquaredErrorCollector
//   SizeInterpreterInterface      (SizeInterpreterInterface.hpp:13) -> GpuGreedySizeInterpreter
//
// Host-memory contract (as the reference): encode returns malloc'd streams the
// caller frees (ComposedRefactor.hpp:41-45); decode / progressive_decode
// return a malloc'd T* the caller frees (ComposedReconstructor.hpp:209,247).
// The adapters therefore copy host <-> device on every call; they exist for
// drop-in compatibility. The throughput path is GpuComposedRefactor /
// GpuComposedReconstructor below (all state resident on the device).
//
// Define PRODM_WITH_REFERENCE_CONCEPTS (and put the reference's include/ on
// the include path) to derive the adapters from the reference's concept base
// classes; otherwise they are free-standing classes with the same signatures.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "prodm_gb300.h"

#ifdef PRODM_WITH_REFERENCE_CONCEPTS
#include "MDR/BitplaneEncoder/BitplaneEncoderInterface.hpp"
#include "MDR/Decomposer/DecomposerInterface.hpp"
#include "MDR/ErrorCollector/ErrorCollectorInterface.hpp"
#include "MDR/Interleaver/InterleaverInterface.hpp"
#include "MDR/SizeInterpreter/SizeInterpreterInterface.hpp"
#define PRODM_BASE(x) : public x
#else
#define PRODM_BASE(x)
#endif

namespace prodm_gb300 {

inline void check(int rc, const char* what) {
    if (rc != PRODM_OK) throw std::runtime_error(std::string(what) + ": " + prodm_last_error_string());
}
inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T> constexpr int dtype_of() { return sizeof(T) == 8 ? PRODM_F64 : PRODM_F32; }

// RAII device buffer
class DeviceBuffer {
  public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t bytes) { resize(bytes); }
    ~DeviceBuffer() { if (p_) cudaFree(p_); }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    void resize(size_t bytes) {
        if (bytes <= cap_) return;
        if (p_) cudaFree(p_);
        p_ = nullptr;
        cuda_check(cudaMalloc(&p_, bytes ? bytes : 1), "cudaMalloc");
        cap_ = bytes;
    }
    void* get() const { return p_; }
    template <class U> U* as() const { return (U*)p_; }

  private:
    void* p_ = nullptr;
    size_t cap_ = 0;
};

inline size_t product(const std::vector<uint32_t>& d) {
    size_t n = 1;
    for (auto x : d) n *= x;
    return n;
}

// ---------------------------------------------------------------------------
// Decomposer: MGARDHierarchicalDecomposer / MGARDOrthoganalDecomposer
// (MGARD.hpp:11-70) on the GPU.
// ---------------------------------------------------------------------------
template <class T, int Basis = PRODM_BASIS_HIERARCHICAL>
class GpuMGARDDecomposer PRODM_BASE(MDR::concepts::DecomposerInterface<T>) {
  public:
    void decompose(T* data, const std::vector<uint32_t>& dims, uint32_t target_level,
                   std::vector<uint32_t> strides = std::vector<uint32_t>()) const {
        run(data, dims, target_level, strides, false);
    }
    void recompose(T* data, const std::vector<uint32_t>& dims, uint32_t target_level,
                   std::vector<uint32_t> strides = std::vector<uint32_t>()) const {
        run(data, dims, target_level, strides, true);
    }
    void print() const { std::printf("GPU MGARD %s decomposer\n", Basis == PRODM_BASIS_HIERARCHICAL ? "hierarchical" : "orthogonal"); }

  private:
    void run(T* data, const std::vector<uint32_t>& dims, uint32_t L, const std::vector<uint32_t>& strides,
             bool inverse) const {
        // the strided array spans dims with the given strides (innermost 1)
        size_t n = product(dims);
        if (!strides.empty()) {
            n = 1;
            for (size_t i = 0; i < dims.size(); i++) n += (size_t)(dims[i] - 1) * strides[i];
        }
        DeviceBuffer d(n * sizeof(T));
        cuda_check(cudaMemcpy(d.get(), data, n * sizeof(T), cudaMemcpyHostToDevice), "H2D");
        const uint32_t* sp = strides.empty() ? nullptr : strides.data();
        int rc = inverse ? prodm_recompose(dtype_of<T>(), d.get(), (int)dims.size(), dims.data(), L, sp, Basis, nullptr, 0,
                                           nullptr)
                         : prodm_decompose(dtype_of<T>(), d.get(), (int)dims.size(), dims.data(), L, sp, Basis, nullptr, 0,
                                           nullptr);
        check(rc, inverse ? "prodm_recompose" : "prodm_decompose");
        cuda_check(cudaMemcpy(data, d.get(), n * sizeof(T), cudaMemcpyDeviceToHost), "D2H");
    }
};
template <class T> using GpuMGARDHierarchicalDecomposer = GpuMGARDDecomposer<T, PRODM_BASIS_HIERARCHICAL>;
template <class T> using GpuMGARDOrthogonalDecomposer = GpuMGARDDecomposer<T, PRODM_BASIS_ORTHOGONAL>;

// ---------------------------------------------------------------------------
// Interleaver: DirectInterleaver (DirectInterleaver.hpp:12-63)
// ---------------------------------------------------------------------------
template <class T>
class GpuDirectInterleaver PRODM_BASE(MDR::concepts::InterleaverInterface<T>) {
  public:
    void interleave(T const* data, const std::vector<uint32_t>& dims, const std::vector<uint32_t>& dims_fine,
                    const std::vector<uint32_t>& dims_coarse, T* buffer,
                    std::vector<uint32_t> strides = std::vector<uint32_t>()) const {
        const size_t n = span(dims, strides), m = count(dims_fine, dims_coarse);
        DeviceBuffer d(n * sizeof(T)), b(m * sizeof(T));
        cuda_check(cudaMemcpy(d.get(), data, n * sizeof(T), cudaMemcpyHostToDevice), "H2D");
        check(prodm_interleave(dtype_of<T>(), d.get(), (int)dims.size(), dims.data(), dims_fine.data(), dims_coarse.data(),
                               b.get(), strides.empty() ? nullptr : strides.data(), nullptr),
              "prodm_interleave");
        cuda_check(cudaMemcpy(buffer, b.get(), m * sizeof(T), cudaMemcpyDeviceToHost), "D2H");
    }
    void reposition(T const* buffer, const std::vector<uint32_t>& dims, const std::vector<uint32_t>& dims_fine,
                    const std::vector<uint32_t>& dims_coarse, T* data,
                    std::vector<uint32_t> strides = std::vector<uint32_t>()) const {
        const size_t n = span(dims, strides), m = count(dims_fine, dims_coarse);
        DeviceBuffer d(n * sizeof(T)), b(m * sizeof(T));
        cuda_check(cudaMemcpy(d.get(), data, n * sizeof(T), cudaMemcpyHostToDevice), "H2D");
        cuda_check(cudaMemcpy(b.get(), buffer, m * sizeof(T), cudaMemcpyHostToDevice), "H2D");
        check(prodm_reposition(dtype_of<T>(), b.get(), (int)dims.size(), dims.data(), dims_fine.data(), dims_coarse.data(),
                               d.get(), strides.empty() ? nullptr : strides.data(), nullptr),
              "prodm_reposition");
        cuda_check(cudaMemcpy(data, d.get(), n * sizeof(T), cudaMemcpyDeviceToHost), "D2H");
    }
    void print() const { std::printf("GPU direct interleaver\n"); }

  private:
    static size_t count(const std::vector<uint32_t>& f, const std::vector<uint32_t>& c) {
        size_t a = product(f), b = product(c);
        return a - b;
    }
    // elements the strided array spans: the reference passes the full array's
    // strides with a smaller box when it reconstructs a coarser level
    // (ComposedReconstructor.hpp:190, :208, :246)
    static size_t span(const std::vector<uint32_t>& dims, const std::vector<uint32_t>& strides) {
        if (strides.empty()) return product(dims);
        size_t n = 1;
        for (size_t i = 0; i < dims.size(); i++) n += (size_t)(dims[i] - 1) * strides[i];
        return n;
    }
};

// ---------------------------------------------------------------------------
// Bitplane encoders: NegaBinaryBPEncoder / GroupedBPEncoder
// ---------------------------------------------------------------------------
template <class T, class S, int Encoder>
class GpuBPEncoder PRODM_BASE(MDR::concepts::BitplaneEncoderInterface<T>) {
    static_assert(sizeof(S) == sizeof(T), "stream words: u32 for float data, u64 for double data");

  public:
    GpuBPEncoder() { check(prodm_decoder_create(&dec_, Encoder, dtype_of<T>()), "prodm_decoder_create"); }
    GpuBPEncoder(const GpuBPEncoder&) : GpuBPEncoder() {}   // decoding state is per object
    GpuBPEncoder& operator=(const GpuBPEncoder&) { return *this; }
    ~GpuBPEncoder() { prodm_decoder_destroy(dec_); }

    std::vector<uint8_t*> encode(T const* data, int32_t n, int32_t exp, uint8_t num_bitplanes,
                                 std::vector<uint32_t>& stream_sizes) const {
        return encode_impl(data, n, exp, num_bitplanes, stream_sizes, nullptr);
    }
    // error-collecting overload (NegaBinaryBPEncoder.hpp:65-125 / GroupedBPEncoder.hpp:76-145)
    std::vector<uint8_t*> encode(T const* data, int32_t n, int32_t exp, uint8_t num_bitplanes,
                                 std::vector<uint32_t>& stream_sizes, std::vector<double>& level_errors) const {
        level_errors.assign(num_bitplanes + 1, 0.0);
        return encode_impl(data, n, exp, num_bitplanes, stream_sizes, &level_errors);
    }
    T* decode(const std::vector<uint8_t const*>& streams, int32_t n, int exp, uint8_t num_bitplanes) {
        // a fresh decoder so that no progressive state leaks into a one-shot decode
        prodm_decoder* d;
        check(prodm_decoder_create(&d, Encoder, dtype_of<T>()), "prodm_decoder_create");
        std::vector<std::vector<uint8_t>> saved;
        saved.swap(rb_);
        T* r = nullptr;
        try {
            r = decode_impl(d, streams, n, exp, 0, num_bitplanes, 0, (int)streams.size());
        } catch (...) {
            rb_.swap(saved);
            prodm_decoder_destroy(d);
            throw;
        }
        rb_.swap(saved);
        prodm_decoder_destroy(d);
        return r;
    }
    // the level's total plane count is not part of the reference signature:
    // set_total_bitplanes() gives it (default: the stream word width)
    T* progressive_decode(const std::vector<uint8_t const*>& streams, int32_t n, int exp, uint8_t starting_bitplane,
                          uint8_t num_bitplanes, int level) {
        return decode_impl(dec_, streams, n, exp, starting_bitplane, num_bitplanes, level, total_planes_);
    }
    void set_total_bitplanes(int b) { total_planes_ = b; }
    void print() const { std::printf("GPU %s bitplane encoder\n", Encoder == PRODM_ENC_NEGABINARY ? "negabinary" : "grouped"); }

  private:
    std::vector<uint8_t*> encode_impl(T const* data, int32_t n, int32_t exp, uint8_t B, std::vector<uint32_t>& sizes,
                                      std::vector<double>* errs) const {
        uint64_t cap = 0;
        check(prodm_encode_bound(Encoder, dtype_of<T>(), (uint64_t)n, B, &cap), "prodm_encode_bound");
        DeviceBuffer d((size_t)n * sizeof(T)), blob(cap + 16), dsz(B * 4), derr((B + 1) * 8);
        cuda_check(cudaMemcpy(d.get(), data, (size_t)n * sizeof(T), cudaMemcpyHostToDevice), "H2D");
        check(prodm_encode(Encoder, dtype_of<T>(), d.get(), (uint64_t)n, exp, B, blob.get(), cap, dsz.as<uint32_t>(),
                           errs ? derr.as<double>() : nullptr, nullptr, 0, nullptr),
              "prodm_encode");
        sizes.assign(B, 0);
        cuda_check(cudaMemcpy(sizes.data(), dsz.get(), B * 4, cudaMemcpyDeviceToHost), "D2H");
        if (errs) cuda_check(cudaMemcpy(errs->data(), derr.get(), (B + 1) * 8, cudaMemcpyDeviceToHost), "D2H");
        std::vector<uint8_t> host(cap);
        size_t total = 0;
        for (auto s : sizes) total += s;
        cuda_check(cudaMemcpy(host.data(), blob.get(), total, cudaMemcpyDeviceToHost), "D2H");
        std::vector<uint8_t*> streams(B);
        size_t off = 0;
        for (int p = 0; p < B; p++) {
            streams[p] = (uint8_t*)std::malloc(sizes[p] ? sizes[p] : 1);
            std::memcpy(streams[p], host.data() + off, sizes[p]);
            off += sizes[p];
        }
        return streams;
    }
    T* decode_impl(prodm_decoder* d, const std::vector<uint8_t const*>& streams, int32_t n, int exp, int s, int num,
                   int level, int total) {
        T* out = (T*)std::malloc((size_t)n * sizeof(T));
        DeviceBuffer dout((size_t)n * sizeof(T));
        if (num == 0) {
            std::memset(out, 0, (size_t)n * sizeof(T));
            return out;
        }
        // stream sizes: fixed for negabinary; for grouped they follow from the
        // per-block recording bitplanes of stream 0's header, which the
        // reference decoder reads the same way (GroupedBPEncoder.hpp:223-230)
        std::vector<uint32_t> sizes(num);
        const uint64_t nb = ((uint64_t)n + 8 * sizeof(S) - 1) / (8 * sizeof(S));
        if (Encoder == PRODM_ENC_NEGABINARY) {
            for (int i = 0; i < num; i++) sizes[i] = (uint32_t)(nb * sizeof(S));
        } else {
            if (s == 0) {
                uint32_t cnt;
                std::memcpy(&cnt, streams[0], 4);
                if ((uint64_t)cnt != nb) throw std::runtime_error("grouped stream header does not match n");
                if ((int)rb_.size() <= level) rb_.resize(level + 1);
                rb_[level].assign(streams[0] + 4, streams[0] + 4 + cnt);
            }
            if ((int)rb_.size() <= level || rb_[level].empty()) throw std::runtime_error("grouped decode: plane 0 first");
            for (int i = 0; i < num; i++) {
                const int p = s + i;
                uint64_t words = 0;
                for (uint8_t r : rb_[level]) words += (r < p ? 1 : 0) + (r == p ? 2 : 0);
                sizes[i] = (uint32_t)(words * sizeof(S) + (p == 0 ? 4 + nb : 0));
            }
        }
        size_t total_bytes = 0;
        for (auto x : sizes) total_bytes += x;
        DeviceBuffer blob(total_bytes + 16);
        std::vector<uint8_t> host(total_bytes);
        size_t off = 0;
        for (int i = 0; i < num; i++) { std::memcpy(host.data() + off, streams[i], sizes[i]); off += sizes[i]; }
        cuda_check(cudaMemcpy(blob.get(), host.data(), total_bytes, cudaMemcpyHostToDevice), "H2D");
        check(prodm_progressive_decode(d, blob.get(), sizes.data(), (uint64_t)n, exp, s, num, level, total, dout.get(), nullptr),
              "prodm_progressive_decode");
        cuda_check(cudaMemcpy(out, dout.get(), (size_t)n * sizeof(T), cudaMemcpyDeviceToHost), "D2H");
        return out;
    }

    prodm_decoder* dec_ = nullptr;
    int total_planes_ = 8 * (int)sizeof(S);
    mutable std::vector<std::vector<uint8_t>> rb_;
};
template <class T, class S> using GpuNegaBinaryBPEncoder = GpuBPEncoder<T, S, PRODM_ENC_NEGABINARY>;
template <class T, class S> using GpuGroupedBPEncoder = GpuBPEncoder<T, S, PRODM_ENC_GROUPED>;

// Stream sizes of every level and plane ([level][plane] bytes), shared between
// adapter objects and their copies. The reference's progressive_decode
// receives stream pointers but no sizes; a per-bit stream's length depends on
// its contents, so GpuPerBitBPEncoder takes the sizes from this table, which a
// GpuGreedySizeInterpreter constructed with the same table fills with the
// metadata sizes it is given on every retrieval.
struct StreamSizeTable {
    std::vector<std::vector<uint32_t>> level;
};

// ---------------------------------------------------------------------------
// Bitplane encoder: PerBitBPEncoder (PerBitBPEncoder.hpp:71-401). S, the
// reference's stream word template argument, does not enter the format.
// progressive_decode takes each stream's size from the next stream's start
// (the retriever hands over one contiguous buffer per level,
// FileRetriever.hpp:69-81); the last stream's size from the shared table when
// it holds the level, else by walking the streams on the host with the
// elements whose sign is known so far.
// ---------------------------------------------------------------------------
template <class T, class S>
class GpuPerBitBPEncoder PRODM_BASE(MDR::concepts::BitplaneEncoderInterface<T>) {
  public:
    explicit GpuPerBitBPEncoder(std::shared_ptr<StreamSizeTable> sizes = nullptr) : table_(std::move(sizes)) {
        check(prodm_decoder_create(&dec_, PRODM_ENC_PERBIT, dtype_of<T>()), "prodm_decoder_create");
    }
    GpuPerBitBPEncoder(const GpuPerBitBPEncoder& o) : GpuPerBitBPEncoder(o.table_) {}   // decoding state is per object
    GpuPerBitBPEncoder& operator=(const GpuPerBitBPEncoder& o) {
        table_ = o.table_;
        return *this;
    }
    ~GpuPerBitBPEncoder() { prodm_decoder_destroy(dec_); }

    std::vector<uint8_t*> encode(T const* data, int32_t n, int32_t exp, uint8_t B,
                                 std::vector<uint32_t>& stream_sizes) const {
        uint64_t cap = 0;
        check(prodm_encode_bound(PRODM_ENC_PERBIT, dtype_of<T>(), (uint64_t)n, B, &cap), "prodm_encode_bound");
        DeviceBuffer d((size_t)n * sizeof(T)), blob(cap + 16), dsz(B * 4);
        cuda_check(cudaMemcpy(d.get(), data, (size_t)n * sizeof(T), cudaMemcpyHostToDevice), "H2D");
        check(prodm_encode(PRODM_ENC_PERBIT, dtype_of<T>(), d.get(), (uint64_t)n, exp, B, blob.get(), cap,
                           dsz.as<uint32_t>(), nullptr, nullptr, 0, nullptr),
              "prodm_encode");
        stream_sizes.assign(B, 0);
        cuda_check(cudaMemcpy(stream_sizes.data(), dsz.get(), B * 4, cudaMemcpyDeviceToHost), "D2H");
        size_t total = 0;
        for (auto x : stream_sizes) total += x;
        std::vector<uint8_t> host(total);
        cuda_check(cudaMemcpy(host.data(), blob.get(), total, cudaMemcpyDeviceToHost), "D2H");
        std::vector<uint8_t*> streams(B);
        size_t off = 0;
        for (int p = 0; p < B; p++) {
            streams[p] = (uint8_t*)std::malloc(stream_sizes[p] ? stream_sizes[p] : 1);
            std::memcpy(streams[p], host.data() + off, stream_sizes[p]);
            off += stream_sizes[p];
        }
        return streams;
    }
    T* decode(const std::vector<uint8_t const*>& streams, int32_t n, int exp, uint8_t num_bitplanes) {
        GpuPerBitBPEncoder fresh(table_);   // no progressive state leaks into a one-shot decode
        return fresh.decode_impl(streams, n, exp, 0, num_bitplanes, 0);
    }
    T* progressive_decode(const std::vector<uint8_t const*>& streams, int32_t n, int exp, uint8_t starting_bitplane,
                          uint8_t num_bitplanes, int level) {
        return decode_impl(streams, n, exp, starting_bitplane, num_bitplanes, level);
    }
    void set_total_bitplanes(int) {}   // per-bit streams carry no level-wide header
    void print() const { std::printf("GPU per-bit bitplane encoder\n"); }

  private:
    // BitDecoder walk (PerBitBPEncoder.hpp:41-67) of planes [s, s+num) for
    // their sizes: one bit per element, plus the sign after a first 1 bit
    std::vector<uint32_t> walk_sizes(const std::vector<uint8_t const*>& streams, int32_t n, int level, int s,
                                     int num) {
        std::vector<uint8_t> known(known_[level]);
        std::vector<uint32_t> sz(num);
        for (int i = 0; i < num; i++) {
            const uint8_t* w = streams[i];
            uint64_t pos = 0;
            for (int32_t j = 0; j < n; j++) {
                const uint64_t b = (w[pos >> 3] >> (pos & 7)) & 1u;
                pos++;
                if (b && !known[j]) { known[j] = 1; pos++; }
            }
            sz[i] = (uint32_t)((pos + 63) / 64 * 8);
        }
        (void)s;
        return sz;
    }
    T* decode_impl(const std::vector<uint8_t const*>& streams, int32_t n, int exp, int s, int num, int level) {
        T* out = (T*)std::malloc((size_t)n * sizeof(T));
        if (num == 0) {
            std::memset(out, 0, (size_t)n * sizeof(T));
            return out;
        }
        if ((int)known_.size() <= level) known_.resize(level + 1);
        if (s == 0 || known_[level].size() != (size_t)n) known_[level].assign(n, 0);
        std::vector<uint32_t> sizes(num, 0);
        bool have = true;
        for (int i = 0; i + 1 < num; i++) {
            const ptrdiff_t d = streams[i + 1] - streams[i];
            if (d <= 0 || d % 8) { have = false; break; }
            sizes[i] = (uint32_t)d;
        }
        const int last = s + num - 1;
        if (have && table_ && level < (int)table_->level.size() && last < (int)table_->level[level].size())
            sizes[num - 1] = table_->level[level][last];
        else
            have = false;
        if (!have) sizes = walk_sizes(streams, n, level, s, num);
        size_t total = 0;
        for (auto x : sizes) total += x;
        DeviceBuffer blob(total + 16), dout((size_t)n * sizeof(T));
        std::vector<uint8_t> host(total);
        size_t off = 0;
        for (int i = 0; i < num; i++) { std::memcpy(host.data() + off, streams[i], sizes[i]); off += sizes[i]; }
        cuda_check(cudaMemcpy(blob.get(), host.data(), total, cudaMemcpyHostToDevice), "H2D");
        // the level's plane count is not part of the signature: room for the most
        check(prodm_progressive_decode(dec_, blob.get(), sizes.data(), (uint64_t)n, exp, s, num, level,
                                       sizeof(T) == 8 ? 63 : 32, dout.get(), nullptr),
              "prodm_progressive_decode");
        cuda_check(cudaMemcpy(out, dout.get(), (size_t)n * sizeof(T), cudaMemcpyDeviceToHost), "D2H");
        // a sign becomes known with an element's first 1 bit: a nonzero contribution
        std::vector<uint8_t>& k = known_[level];
        for (int32_t j = 0; j < n; j++) k[j] |= out[j] != (T)0;
        return out;
    }

    prodm_decoder* dec_ = nullptr;
    std::shared_ptr<StreamSizeTable> table_;
    std::vector<std::vector<uint8_t>> known_;
};

// ---------------------------------------------------------------------------
// Lossless stage: AdaptiveLevelCompressor's rule (AdaptiveLevelCompressor.hpp:
// 13-60) with this library's GPU codec ZCB instead of zstd (files of the
// reference's zstd stage are not readable with it)
// ---------------------------------------------------------------------------
class GpuAdaptiveLevelCompressor PRODM_BASE(MDR::concepts::LevelCompressorInterface) {
  public:
    explicit GpuAdaptiveLevelCompressor(int latter = 26) : latter_(latter) {}
    GpuAdaptiveLevelCompressor(const GpuAdaptiveLevelCompressor& o) : latter_(o.latter_) {}
    GpuAdaptiveLevelCompressor& operator=(const GpuAdaptiveLevelCompressor& o) {
        latter_ = o.latter_;
        return *this;
    }
    ~GpuAdaptiveLevelCompressor() { decompress_release(); }

    uint8_t compress_level(std::vector<uint8_t*>& streams, std::vector<uint32_t>& stream_sizes) const {
        const int B = (int)stream_sizes.size();
        size_t total = 0;
        for (auto x : stream_sizes) total += x;
        std::vector<uint8_t> host(total);
        size_t o = 0;
        for (int p = 0; p < B; p++) { std::memcpy(host.data() + o, streams[p], stream_sizes[p]); o += stream_sizes[p]; }
        uint64_t cap = 0;
        check(prodm_lossless_compress_bound(stream_sizes.data(), B, &cap), "prodm_lossless_compress_bound");
        DeviceBuffer in(total + 16), out(cap + 16);
        cuda_check(cudaMemcpy(in.get(), host.data(), total, cudaMemcpyHostToDevice), "H2D");
        std::vector<uint32_t> osz(B);
        int stop = 0;
        check(prodm_lossless_compress_level(in.get(), stream_sizes.data(), B, latter_, out.get(), cap, osz.data(), &stop,
                                            nullptr),
              "prodm_lossless_compress_level");
        size_t ot = 0;
        for (auto x : osz) ot += x;
        std::vector<uint8_t> res(ot);
        cuda_check(cudaMemcpy(res.data(), out.get(), ot, cudaMemcpyDeviceToHost), "D2H");
        o = 0;
        for (int p = 0; p < B; p++) {   // overwrite and free the original streams (LevelCompressorInterface.hpp:13)
            std::free(streams[p]);
            streams[p] = (uint8_t*)std::malloc(osz[p] ? osz[p] : 1);
            std::memcpy(streams[p], res.data() + o, osz[p]);
            stream_sizes[p] = osz[p];
            o += osz[p];
        }
        return (uint8_t)stop;
    }
    void decompress_level(std::vector<const uint8_t*>& streams, const std::vector<uint32_t>& stream_sizes,
                          uint8_t starting_bitplane, uint8_t num_bitplanes, uint8_t stopping_index) {
        if (!num_bitplanes) return;
        std::vector<uint32_t> sz(num_bitplanes);
        size_t total = 0, raw = 0;
        for (int i = 0; i < num_bitplanes; i++) {
            const int p = starting_bitplane + i;
            sz[i] = stream_sizes.at(p);
            total += sz[i];
            if (p <= stopping_index || p >= latter_) {   // the raw length leads a compressed stream
                uint64_t n = 0;
                if (sz[i] >= 8) std::memcpy(&n, streams[i], 8);
                raw += n;
            } else {
                raw += sz[i];
            }
        }
        std::vector<uint8_t> host(total);
        size_t o = 0;
        for (int i = 0; i < num_bitplanes; i++) { std::memcpy(host.data() + o, streams[i], sz[i]); o += sz[i]; }
        DeviceBuffer in(total + 16), out(raw + 16);
        cuda_check(cudaMemcpy(in.get(), host.data(), total, cudaMemcpyHostToDevice), "H2D");
        std::vector<uint32_t> rsz(num_bitplanes);
        check(prodm_lossless_decompress_level(in.get(), sz.data(), starting_bitplane, num_bitplanes, stopping_index,
                                              latter_, out.get(), raw, rsz.data(), nullptr),
              "prodm_lossless_decompress_level");
        std::vector<uint8_t> res(raw);
        cuda_check(cudaMemcpy(res.data(), out.get(), raw, cudaMemcpyDeviceToHost), "D2H");
        o = 0;
        for (int i = 0; i < num_bitplanes; i++) {
            uint8_t* b = (uint8_t*)std::malloc(rsz[i] ? rsz[i] : 1);
            std::memcpy(b, res.data() + o, rsz[i]);
            o += rsz[i];
            buffer_.push_back(b);
            streams[i] = b;
        }
    }
    void decompress_release() {
        for (auto* b : buffer_) std::free(b);
        buffer_.clear();
    }
    void print() const { std::printf("GPU adaptive level compressor (ZCB codec)\n"); }

  private:
    int latter_;
    std::vector<uint8_t*> buffer_;
};

// ---------------------------------------------------------------------------
// Error collectors (MaxErrorCollector.hpp:14-25, SquaredErrorCollector.hpp:54-96)
// ---------------------------------------------------------------------------
template <class T>
class GpuMaxErrorCollector PRODM_BASE(MDR::concepts::ErrorCollectorInterface<T>) {
  public:
    std::vector<double> collect_level_error(T const* data, size_t n, int num_bitplanes, T max_level_error) const {
        (void)data; (void)n;
        std::vector<double> out(num_bitplanes + 1);
        check(prodm_collect_max(dtype_of<T>(), (double)max_level_error, num_bitplanes, out.data()), "prodm_collect_max");
        return out;
    }
    void print() const { std::printf("GPU max error collector\n"); }
};

template <class T>
class GpuSquaredErrorCollector PRODM_BASE(MDR::concepts::ErrorCollectorInterface<T>) {
  public:
    std::vector<double> collect_level_error(T const* data, size_t n, int num_bitplanes, T max_level_error) const {
        DeviceBuffer d(n * sizeof(T)), o((num_bitplanes + 1) * 8);
        cuda_check(cudaMemcpy(d.get(), data, n * sizeof(T), cudaMemcpyHostToDevice), "H2D");
        check(prodm_collect_squared(dtype_of<T>(), d.get(), n, num_bitplanes, (double)max_level_error, o.as<double>(),
                                    nullptr, 0, nullptr),
              "prodm_collect_squared");
        std::vector<double> out(num_bitplanes + 1);
        cuda_check(cudaMemcpy(out.data(), o.get(), out.size() * 8, cudaMemcpyDeviceToHost), "D2H");
        return out;
    }
    void print() const { std::printf("GPU squared error collector\n"); }
};

// ---------------------------------------------------------------------------
// Size interpreters (GreedyBasedSizeInterpreter.hpp:28-248) with the
// estimator selected by kind (MaxErrorEstimator.hpp / SquaredErrorEstimator.hpp)
// ---------------------------------------------------------------------------
template <class T, int Interp, int Estimator>
class GpuGreedySizeInterpreter PRODM_BASE(MDR::concepts::SizeInterpreterInterface) {
  public:
    explicit GpuGreedySizeInterpreter(int ndims = 3, double s = 0.0) : ndims_(ndims), s_(s) {}
    template <class E>
    explicit GpuGreedySizeInterpreter(const E&, int ndims = 3, double s = 0.0) : ndims_(ndims), s_(s) {}
    // publishes the stream sizes it is given into `sizes` (for GpuPerBitBPEncoder)
    template <class E>
    GpuGreedySizeInterpreter(const E&, std::shared_ptr<StreamSizeTable> sizes, int ndims = 3, double s = 0.0)
        : ndims_(ndims), s_(s), table_(std::move(sizes)) {}
    std::vector<uint32_t> interpret_retrieve_size(const std::vector<std::vector<uint32_t>>& level_sizes,
                                                  const std::vector<std::vector<double>>& level_errors,
                                                  double tolerance, std::vector<uint8_t>& index) const {
        if (table_) table_->level = level_sizes;
        const int nl = (int)level_sizes.size();
        const int B = (int)level_sizes[0].size();
        std::vector<uint32_t> sz(nl * B);
        std::vector<double> er(nl * (B + 1));
        for (int l = 0; l < nl; l++) {
            std::memcpy(sz.data() + l * B, level_sizes[l].data(), B * 4);
            std::memcpy(er.data() + l * (B + 1), level_errors[l].data(), (B + 1) * 8);
        }
        DeviceBuffer dsz(sz.size() * 4), der(er.size() * 8), didx(nl), drs(nl * 4);
        cuda_check(cudaMemcpy(dsz.get(), sz.data(), sz.size() * 4, cudaMemcpyHostToDevice), "H2D");
        cuda_check(cudaMemcpy(der.get(), er.data(), er.size() * 8, cudaMemcpyHostToDevice), "H2D");
        cuda_check(cudaMemcpy(didx.get(), index.data(), nl, cudaMemcpyHostToDevice), "H2D");
        check(prodm_interpret(Interp, Estimator, dtype_of<T>(), ndims_, nl - 1, s_, nl, B, dsz.as<uint32_t>(),
                              der.as<double>(), tolerance, didx.as<uint8_t>(), drs.as<uint32_t>(), nullptr),
              "prodm_interpret");
        std::vector<uint32_t> rs(nl);
        cuda_check(cudaMemcpy(index.data(), didx.get(), nl, cudaMemcpyDeviceToHost), "D2H");
        cuda_check(cudaMemcpy(rs.data(), drs.get(), nl * 4, cudaMemcpyDeviceToHost), "D2H");
        return rs;
    }
    void print() const { std::printf("GPU greedy size interpreter\n"); }

  private:
    int ndims_;
    double s_;
    std::shared_ptr<StreamSizeTable> table_;
};

// ---------------------------------------------------------------------------
// Device-resident composed refactor / reconstructor with the public API of
// ComposedRefactor (ComposedRefactor.hpp:21-67) and ComposedReconstructor
// (ComposedReconstructor.hpp:23-174). Level files and metadata use the
// reference's on-disk format (FileWriter.hpp:13-39), so files written here
// load into the reference reconstructor and vice versa (the metadata carries
// an extra squared-error table after the reference fields).
// ---------------------------------------------------------------------------
template <class T>
class GpuComposedRefactor {
  public:
    GpuComposedRefactor(int encoder, int basis, int collector, std::string metadata_file,
                        std::vector<std::string> level_files)
        : enc_(encoder), basis_(basis), col_(collector), meta_(std::move(metadata_file)), files_(std::move(level_files)) {}
    // the lossless stage (AdaptiveLevelCompressor's rule, ZCB codec); < 0: none
    void set_lossless(int latter_index) { latter_ = latter_index; }
    ~GpuComposedRefactor() { if (h_) prodm_mdr_destroy(h_); }

    void refactor(T const* data, const std::vector<uint32_t>& dims, uint8_t target_level, uint8_t num_bitplanes) {
        prodm_config c{};
        c.dtype = dtype_of<T>();
        c.ndims = (int)dims.size();
        for (size_t i = 0; i < dims.size(); i++) c.dims[i] = dims[i];
        c.target_level = target_level;
        c.num_bitplanes = num_bitplanes;
        c.encoder = enc_;
        c.basis = basis_;
        c.collector = col_;
        if (h_) prodm_mdr_destroy(h_);
        check(prodm_mdr_create(&h_, &c), "prodm_mdr_create");
        const size_t n = product(dims);
        DeviceBuffer d(n * sizeof(T));
        cuda_check(cudaMemcpy(d.get(), data, n * sizeof(T), cudaMemcpyHostToDevice), "H2D");
        check(prodm_mdr_set_lossless(h_, latter_, nullptr), "prodm_mdr_set_lossless");
        check(prodm_mdr_refactor(h_, d.get(), nullptr), "prodm_mdr_refactor");
        for (int l = 0; l <= target_level; l++)
            check(prodm_mdr_write_level_file(h_, l, files_.at(l).c_str(), nullptr), "prodm_mdr_write_level_file");
        write_metadata();
    }
    void write_metadata() const {
        size_t len = 0;
        check(prodm_mdr_metadata(h_, nullptr, 0, &len, nullptr), "prodm_mdr_metadata");
        std::vector<uint8_t> buf(len);
        check(prodm_mdr_metadata(h_, buf.data(), len, &len, nullptr), "prodm_mdr_metadata");
        write_file(meta_, buf);
    }
    void print() const { std::printf("GPU composed refactor\n"); }

  private:
    static void write_file(const std::string& f, const std::vector<uint8_t>& b) {
        FILE* fp = std::fopen(f.c_str(), "wb");
        if (!fp) throw std::runtime_error("cannot write " + f);
        std::fwrite(b.data(), 1, b.size(), fp);
        std::fclose(fp);
    }
    int enc_, basis_, col_;
    int latter_ = -1;
    std::string meta_;
    std::vector<std::string> files_;
    prodm_mdr* h_ = nullptr;
};

template <class T>
class GpuComposedReconstructor {
  public:
    GpuComposedReconstructor(int encoder, int basis, int interpreter, int estimator, std::string metadata_file,
                             std::vector<std::string> level_files, double s = 0.0)
        : enc_(encoder), basis_(basis), interp_(interpreter), est_(estimator), s_(s), meta_(std::move(metadata_file)),
          files_(std::move(level_files)) {}
    ~GpuComposedReconstructor() { if (h_) prodm_mdr_destroy(h_); }

    void load_metadata() {
        std::vector<uint8_t> m = read_file(meta_);
        const int nd = m.at(0);
        dims_.assign(nd, 0);
        std::memcpy(dims_.data(), m.data() + 1, 4 * nd);
        const int nl = m.at(1 + 4 * nd);
        const uint8_t* p = m.data() + 2 + 4 * nd + nl * sizeof(T);
        uint32_t B;
        std::memcpy(&B, p, 4);
        prodm_config c{};
        c.dtype = dtype_of<T>();
        c.ndims = nd;
        for (int i = 0; i < nd; i++) c.dims[i] = dims_[i];
        c.target_level = nl - 1;
        c.num_bitplanes = (int)B;
        c.encoder = enc_;
        c.basis = basis_;
        // the squared-error table of the metadata feeds the L2 estimators; the
        // per-bit encoder is used with the max collector only
        c.collector = enc_ == PRODM_ENC_PERBIT ? PRODM_COLLECT_MAX : PRODM_COLLECT_SQUARED;
        if (h_) prodm_mdr_destroy(h_);
        check(prodm_mdr_create(&h_, &c), "prodm_mdr_create");
        check(prodm_mdr_load_metadata(h_, m.data(), m.size(), nullptr), "prodm_mdr_load_metadata");
        nl_ = nl;
        B_ = (int)B;
        sizes_.assign(nl * B, 0);
        check(prodm_mdr_level_info(h_, sizes_.data(), nullptr, nullptr, nullptr), "prodm_mdr_level_info");
        loaded_.assign(nl, 0);
        out_.resize(product(dims_) * sizeof(T));
        host_.assign(product(dims_), (T)0);
    }
    T* reconstruct(double tolerance) { return progressive_reconstruct(tolerance); }
    T* progressive_reconstruct(double tolerance) {
        check(prodm_mdr_interpret(h_, tolerance, interp_, est_, s_, nullptr), "prodm_mdr_interpret");
        std::vector<uint8_t> idx(nl_);
        check(prodm_mdr_get_index(h_, idx.data(), nullptr), "prodm_mdr_get_index");
        retrieved_ = 0;
        for (int l = 0; l < nl_; l++) {
            uint64_t need = 0;
            for (int p = 0; p < idx[l]; p++) need += sizes_[l * B_ + p];
            if (need > loaded_[l]) {   // ConcatLevelFileRetriever: read the next bytes of the level file
                check(prodm_mdr_load_level_file(h_, l, files_.at(l).c_str(), loaded_[l], loaded_[l], need - loaded_[l],
                                                nullptr),
                      "prodm_mdr_load_level_file");
                loaded_[l] = need;
            }
            retrieved_ += loaded_[l];
        }
        check(prodm_mdr_reconstruct(h_, out_.get(), nullptr), "prodm_mdr_reconstruct");
        cuda_check(cudaMemcpy(host_.data(), out_.get(), host_.size() * sizeof(T), cudaMemcpyDeviceToHost), "D2H");
        return host_.data();
    }
    const std::vector<uint32_t>& get_dimensions() { return dims_; }
    size_t get_retrieved_size() { return retrieved_; }
    void print() const { std::printf("GPU composed reconstructor\n"); }

  private:
    static std::vector<uint8_t> read_file(const std::string& f) {
        FILE* fp = std::fopen(f.c_str(), "rb");
        if (!fp) throw std::runtime_error("cannot read " + f);
        std::fseek(fp, 0, SEEK_END);
        long n = std::ftell(fp);
        std::rewind(fp);
        std::vector<uint8_t> b(n);
        if (n && std::fread(b.data(), 1, n, fp) != (size_t)n) throw std::runtime_error("short read " + f);
        std::fclose(fp);
        return b;
    }
    int enc_, basis_, interp_, est_;
    double s_;
    std::string meta_;
    std::vector<std::string> files_;
    prodm_mdr* h_ = nullptr;
    std::vector<uint32_t> dims_, sizes_;
    int nl_ = 0, B_ = 0;
    std::vector<uint64_t> loaded_;
    DeviceBuffer out_;
    std::vector<T> host_;
    size_t retrieved_ = 0;
};

}  // namespace prodm_gb300
