// Level-file I/O for the device-resident handle: byte ranges of the
// reference's level files (ConcatLevelFileWriter / ConcatLevelFileRetriever,
// FileWriter.hpp:13-39, FileRetriever.hpp:15-35) read straight into device
// memory, and level files written from it.
//
// Reads go through cuFile (GPUDirect Storage; libcufile is opened at run time)
// into device staging buffers when its driver opens and the file registers,
// else through pread into two pinned host buffers whose asynchronous copies
// overlap the next read. Either way each staged chunk enters the handle's
// ordinary loading path (the lossless stage's stored bytes included).
#include <dlfcn.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include <cufile.h>

#include "common.cuh"
#include "kernels.cuh"

namespace prodm {
namespace {

struct CuFileApi {
    bool ok = false;
    decltype(&cuFileDriverOpen) driver_open = nullptr;
    decltype(&cuFileHandleRegister) reg = nullptr;
    decltype(&cuFileHandleDeregister) dereg = nullptr;
    decltype(&cuFileRead) read = nullptr;
};

CuFileApi& cufile() {
    static CuFileApi api;
    static std::once_flag once;
    std::call_once(once, [] {
        // cuFile writes its log into the working directory unless told otherwise
        setenv("CUFILE_LOGFILE_PATH", "/tmp/prodm_gb300_cufile.log", 0);
        void* h = dlopen("libcufile.so.0", RTLD_NOW | RTLD_LOCAL);
        if (!h) h = dlopen("libcufile.so", RTLD_NOW | RTLD_LOCAL);
        if (!h) return;
        api.driver_open = (decltype(api.driver_open))dlsym(h, "cuFileDriverOpen");
        api.reg = (decltype(api.reg))dlsym(h, "cuFileHandleRegister");
        api.dereg = (decltype(api.dereg))dlsym(h, "cuFileHandleDeregister");
        api.read = (decltype(api.read))dlsym(h, "cuFileRead");
        if (!api.driver_open || !api.reg || !api.dereg || !api.read) return;
        const CUfileError_t e = api.driver_open();
        api.ok = e.err == CU_FILE_SUCCESS;
    });
    return api;
}

constexpr uint64_t kChunk = 16ull << 20;

// file systems on which cuFile refused to register a file: not tried again
std::mutex g_noreg_mu;
std::set<dev_t> g_noreg;

}  // namespace

// per-handle staging (two device and two pinned buffers of kChunk bytes, and
// the events that guard their reuse)
struct FileStaging {
    void* dev[2] = {nullptr, nullptr};
    void* host[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    int mode = -1;   // 1 cuFile, 0 pinned, -1 no read yet
    ~FileStaging() {
        for (int i = 0; i < 2; i++) {
            if (done[i]) cudaEventSynchronize(done[i]), cudaEventDestroy(done[i]);
            if (dev[i]) cudaFree(dev[i]);
            if (host[i]) cudaFreeHost(host[i]);
        }
    }
};

void file_staging_free(FileStaging* s) { delete s; }
int file_staging_mode(const FileStaging* s) { return s->mode; }

// read file bytes [file_off, file_off + bytes) into the handle's level data at
// level_off through `sink` (the handle's loader: device or pinned host source)
int read_file_range(FileStaging*& fs, const char* path, uint64_t file_off, uint64_t bytes,
                    const std::function<int(const void*, uint64_t, uint64_t, int)>& sink, cudaStream_t st,
                    int* mode_out) {
    if (!fs) fs = new FileStaging();
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return fail(PRODM_EINVAL, std::string("cannot open ") + path);
    struct Closer {
        int fd;
        ~Closer() { close(fd); }
    } closer{fd};
    for (int i = 0; i < 2; i++)
        if (!fs->done[i]) PRODM_CUDA(cudaEventCreateWithFlags(&fs->done[i], cudaEventDisableTiming));
    CuFileApi& cf = cufile();
    CUfileHandle_t fh{};
    bool direct = false;
    struct stat sb;
    const bool have_dev = fstat(fd, &sb) == 0;
    bool refused = false;
    if (have_dev) {
        std::lock_guard<std::mutex> g(g_noreg_mu);
        refused = g_noreg.count(sb.st_dev) != 0;
    }
    if (cf.ok && !refused) {
        CUfileDescr_t d;
        std::memset(&d, 0, sizeof(d));
        d.handle.fd = fd;
        d.type = CU_FILE_HANDLE_TYPE_OPAQUE_FD;
        direct = cf.reg(&fh, &d).err == CU_FILE_SUCCESS;
        if (!direct && have_dev) {
            std::lock_guard<std::mutex> g(g_noreg_mu);
            g_noreg.insert(sb.st_dev);
        }
    }
    fs->mode = direct ? 1 : 0;
    if (mode_out) *mode_out = fs->mode;
    int rc = PRODM_OK;
    uint64_t done = 0;
    int k = 0;
    while (done < bytes && rc == PRODM_OK) {
        const uint64_t n = bytes - done < kChunk ? bytes - done : kChunk;
        const int b = k & 1;
        cudaError_t e = cudaEventSynchronize(fs->done[b]);   // the buffer's previous copy has finished
        if (e != cudaSuccess) { rc = cuda_status(e, "file staging"); break; }
        if (direct) {
            if (!fs->dev[b] && (e = cudaMalloc(&fs->dev[b], kChunk)) != cudaSuccess) { rc = cuda_status(e, "cudaMalloc"); break; }
            const ssize_t got = cf.read(fh, fs->dev[b], n, (off_t)(file_off + done), 0);
            if (got != (ssize_t)n) { rc = fail(PRODM_EINVAL, std::string("short read of ") + path); break; }
            rc = sink(fs->dev[b], done, n, 0);
        } else {
            if (!fs->host[b] && (e = cudaMallocHost(&fs->host[b], kChunk)) != cudaSuccess) { rc = cuda_status(e, "cudaMallocHost"); break; }
            uint64_t r = 0;
            while (r < n) {
                const ssize_t got = pread(fd, (uint8_t*)fs->host[b] + r, n - r, (off_t)(file_off + done + r));
                if (got <= 0) break;
                r += (uint64_t)got;
            }
            if (r != n) { rc = fail(PRODM_EINVAL, std::string("short read of ") + path); break; }
            rc = sink(fs->host[b], done, n, 1);
        }
        if (rc == PRODM_OK && (e = cudaEventRecord(fs->done[b], st)) != cudaSuccess) rc = cuda_status(e, "cudaEventRecord");
        done += n;
        k++;
    }
    if (direct) cf.dereg(fh);
    return rc;
}

}  // namespace prodm
