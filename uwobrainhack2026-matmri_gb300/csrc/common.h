// Shared host/device helpers for libmatmri_gb300 (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <stdexcept>
#include <vector>

#include "../../include/matmri_gb300.h"

namespace mmr {

// ---------------------------------------------------------------- errors ----
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& m);

#define MMR_THROW(code, ...)                                                   \
    do {                                                                       \
        char _b[512];                                                          \
        snprintf(_b, sizeof(_b), __VA_ARGS__);                                 \
        throw ::mmr::Error((code), std::string(_b));                           \
    } while (0)

#define MMR_CUDA(call)                                                         \
    do {                                                                       \
        cudaError_t _e = (call);                                               \
        if (_e != cudaSuccess) {                                               \
            (void)cudaGetLastError();                                          \
            MMR_THROW(_e == cudaErrorMemoryAllocation ? MMR_ERR_NOMEM : MMR_ERR_CUDA, \
                      "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e),  \
                      __FILE__, __LINE__);                                     \
        }                                                                      \
    } while (0)

#define MMR_REQUIRE(cond, ...)                                                 \
    do {                                                                       \
        if (!(cond)) MMR_THROW(MMR_ERR_BADARG, __VA_ARGS__);                   \
    } while (0)

// Runs `body` and converts exceptions into a status code + thread-local message.
template <class F>
int guarded(F&& body) {
    try {
        body();
        return MMR_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return MMR_ERR_NOMEM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return MMR_ERR_CUDA;
    }
}

// ------------------------------------------------- launch counting / profiling ----
// Kernels launched by the library: eager launches are counted as they are
// issued; launches recorded into a graph are counted when the graph replays.
void note_launch();
void set_capturing(bool on);
void add_launches(uint64_t n);
// Stage profiler: when active, prof_mark() records a CUDA event on `st`
// tagged with the stage that starts there (stage < 0 closes the last one).
void prof_mark(int stage, cudaStream_t st);
void prof_begin();
void prof_end(double* ms, int* count, int nstage);

inline void check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) MMR_THROW(MMR_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
    note_launch();
}

// ------------------------------------------------ programmatic dependent launch ----
// A kernel launched with launch_dependent() may be scheduled while the kernel before it
// on the stream is still finishing (its CTAs fill the SMs that the tail frees).  Every
// such kernel calls pdl_wait() before it touches global memory, which returns once the
// previous grid has completed and its writes are visible; pdl_trigger() then lets the
// next kernel start launching once all of this grid's CTAs are running.  Both are
// no-ops in a kernel launched the ordinary way.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... KArgs, class... Args>
void launch_dependent(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        MMR_THROW(MMR_ERR_CUDA, "launch failed: %s", cudaGetErrorString(e));
    }
    note_launch();
}

// ----------------------------------------------------------- device buffer ----
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    // Grows (never shrinks); contents are not preserved.
    void ensure(size_t b) {
        if (b <= bytes) return;
        release();
        if (b == 0) return;
        MMR_CUDA(cudaMalloc(&p, b));
        bytes = b;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
    template <class T> void upload(const std::vector<T>& v) {
        ensure(v.size() * sizeof(T));
        if (!v.empty()) MMR_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    }
};

// True when `ptr` is device-accessible memory (cudaMalloc / managed).
bool is_device_ptr(const void* ptr);

// Host <-> device staging for entry points that accept host or device pointers.
struct Staged {
    const void* user = nullptr;
    bool host = false;
    DevBuf buf;
    void* dev = nullptr;
};
// Input: returns a device pointer holding `bytes` of `user` data.
const void* stage_in(Staged& s, const void* user, size_t bytes, cudaStream_t st);
// Output: returns a device pointer to write into; call finish_out afterwards.
void* stage_out(Staged& s, void* user, size_t bytes);
void finish_out(Staged& s, size_t bytes, cudaStream_t st);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int device_sm_count();
int device_smem_optin();

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace mmr
