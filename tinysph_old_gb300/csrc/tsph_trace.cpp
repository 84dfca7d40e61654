// Kernel timeline of the library's own launches through CUPTI's activity
// API: GPU start and end timestamps of every kernel, including kernels
// replayed from a CUDA graph, where per-launch CUDA events cannot be placed.
// Used by the benchmark to split a graph step's time by kernel; not part of
// the time step itself (libtsph_trace.so, optional: built only where CUPTI
// is installed).
//
//   tsph_trace_start()   enable kernel activity records, clear the list
//   tsph_trace_stop()    flush the records and disable them
//   tsph_trace_count()   records collected
//   tsph_trace_get(i, name, cap, &start, &end, &stream)   record i (ns)

#include <cupti.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace {

struct KernelRecord {
    std::string name;
    uint64_t start, end;
    uint32_t stream;
};

std::mutex g_mu;
std::vector<KernelRecord> g_records;
bool g_registered = false;
constexpr size_t kBufBytes = 8u << 20;

void CUPTIAPI buffer_requested(uint8_t **buffer, size_t *size, size_t *max_records) {
    *buffer = static_cast<uint8_t *>(std::aligned_alloc(64, kBufBytes));
    *size = *buffer ? kBufBytes : 0;
    *max_records = 0;
}

void CUPTIAPI buffer_completed(CUcontext, uint32_t, uint8_t *buffer, size_t, size_t valid) {
    CUpti_Activity *rec = nullptr;
    std::lock_guard<std::mutex> lock(g_mu);
    while (cuptiActivityGetNextRecord(buffer, valid, &rec) == CUPTI_SUCCESS) {
        if (rec->kind != CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL) continue;
        const auto *k = reinterpret_cast<const CUpti_ActivityKernel10 *>(rec);
        g_records.push_back({k->name ? std::string(k->name) : std::string(), k->start, k->end,
                             k->streamId});
    }
    std::free(buffer);
}

}  // namespace

extern "C" {

int tsph_trace_start(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_records.clear();
    if (!g_registered) {
        if (cuptiActivityRegisterCallbacks(buffer_requested, buffer_completed) != CUPTI_SUCCESS)
            return 1;
        g_registered = true;
    }
    return cuptiActivityEnable(CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL) == CUPTI_SUCCESS ? 0 : 2;
}

int tsph_trace_stop(void) {
    // the caller has synchronised the device; flush every buffer, complete or not
    if (cuptiActivityFlushAll(1) != CUPTI_SUCCESS) return 1;
    return cuptiActivityDisable(CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL) == CUPTI_SUCCESS ? 0 : 2;
}

int tsph_trace_count(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    return (int)g_records.size();
}

int tsph_trace_get(int i, char *name, int cap, unsigned long long *start, unsigned long long *end,
                   unsigned int *stream) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (i < 0 || i >= (int)g_records.size() || !name || cap < 1) return 1;
    const KernelRecord &r = g_records[(size_t)i];
    std::strncpy(name, r.name.c_str(), (size_t)cap - 1);
    name[cap - 1] = '\0';
    *start = r.start;
    *end = r.end;
    *stream = r.stream;
    return 0;
}

}  // extern "C"
