// Library-wide helpers: error state, pointer staging, device queries, ABI info.
#include <atomic>

#include "common.h"

namespace mmr {

static thread_local std::string g_last_error;

void set_last_error(const std::string& m) { g_last_error = m; }

bool is_device_ptr(const void* ptr) {
    if (!ptr) return false;
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, ptr);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

const void* stage_in(Staged& s, const void* user, size_t bytes, cudaStream_t st) {
    s.user = user;
    if (is_device_ptr(user)) {
        s.host = false;
        return user;
    }
    s.host = true;
    s.buf.ensure(bytes);
    MMR_CUDA(cudaMemcpyAsync(s.buf.p, user, bytes, cudaMemcpyHostToDevice, st));
    return s.buf.p;
}

void* stage_out(Staged& s, void* user, size_t bytes) {
    s.user = user;
    if (is_device_ptr(user)) {
        s.host = false;
        s.dev = user;
        return user;
    }
    s.host = true;
    s.buf.ensure(bytes);
    s.dev = s.buf.p;
    return s.dev;
}

void finish_out(Staged& s, size_t bytes, cudaStream_t st) {
    if (!s.host) return;
    MMR_CUDA(cudaMemcpyAsync(const_cast<void*>(s.user), s.dev, bytes, cudaMemcpyDeviceToHost, st));
    MMR_CUDA(cudaStreamSynchronize(st));
}

static std::atomic<uint64_t> g_launches{0};
static thread_local bool g_capturing = false;

void note_launch() {
    if (!g_capturing) g_launches.fetch_add(1, std::memory_order_relaxed);
}
void set_capturing(bool on) { g_capturing = on; }
void add_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

struct Prof {
    std::vector<cudaEvent_t> ev;
    std::vector<int> stage;
};
static thread_local Prof* g_prof = nullptr;

void prof_mark(int stage, cudaStream_t st) {
    if (!g_prof || g_capturing) return;
    cudaEvent_t e;
    MMR_CUDA(cudaEventCreate(&e));
    MMR_CUDA(cudaEventRecord(e, st));
    g_prof->ev.push_back(e);
    g_prof->stage.push_back(stage);
}

void prof_begin() {
    delete g_prof;
    g_prof = new Prof();
}

// Sums elapsed time per stage (ms) and counts the intervals; frees the events.
void prof_end(double* ms, int* count, int nstage) {
    Prof* p = g_prof;
    g_prof = nullptr;
    if (!p) return;
    for (int i = 0; i < nstage; ++i) { ms[i] = 0; count[i] = 0; }
    if (!p->ev.empty()) MMR_CUDA(cudaEventSynchronize(p->ev.back()));
    for (size_t i = 0; i + 1 < p->ev.size(); ++i) {
        const int s = p->stage[i];
        if (s < 0 || s >= nstage) continue;
        float t = 0;
        MMR_CUDA(cudaEventElapsedTime(&t, p->ev[i], p->ev[i + 1]));
        ms[s] += t;
        count[s] += 1;
    }
    for (auto e : p->ev) cudaEventDestroy(e);
    delete p;
}

static int g_sm = -1, g_smem = -1;

int device_sm_count() {
    if (g_sm < 0) {
        int dev = 0;
        MMR_CUDA(cudaGetDevice(&dev));
        MMR_CUDA(cudaDeviceGetAttribute(&g_sm, cudaDevAttrMultiProcessorCount, dev));
    }
    return g_sm;
}

int device_smem_optin() {
    if (g_smem < 0) {
        int dev = 0;
        MMR_CUDA(cudaGetDevice(&dev));
        MMR_CUDA(cudaDeviceGetAttribute(&g_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    }
    return g_smem;
}

}  // namespace mmr

extern "C" int mmr_abi_version(void) { return MMR_ABI_VERSION; }

extern "C" int mmr_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return MMR_ERR_BADARG;
    std::string& m = mmr::g_last_error;
    size_t n = m.size() < len - 1 ? m.size() : len - 1;
    memcpy(buf, m.data(), n);
    buf[n] = '\0';
    return MMR_OK;
}

extern "C" int mmr_device_info(int* sm_count, int* smem_optin_bytes, int* cc_major, int* cc_minor) {
    return mmr::guarded([&] {
        int dev = 0;
        MMR_CUDA(cudaGetDevice(&dev));
        if (sm_count) *sm_count = mmr::device_sm_count();
        if (smem_optin_bytes) *smem_optin_bytes = mmr::device_smem_optin();
        if (cc_major) MMR_CUDA(cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev));
        if (cc_minor) MMR_CUDA(cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
    });
}

extern "C" int mmr_kernel_launches(uint64_t* count) {
    return mmr::guarded([&] {
        MMR_REQUIRE(count, "NULL argument");
        *count = mmr::g_launches.load();
    });
}
