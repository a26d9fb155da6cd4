// Runtime services of the C-ABI library (defined in sde_api.cu) for entry
// points defined in other translation units: the per-device stream, scratch
// cache, kernel timing events and the last-error text.
#pragma once
#include <cstddef>
#include <mutex>

#include <cuda_runtime.h>

namespace sdegpu {

struct RtCall {
    cudaStream_t st;      // the library's stream on the current device
    int sms;              // its multiprocessor count
    bool timing;          // sde_timing enabled: record ev0/ev1 around the main kernel
    cudaEvent_t ev0, ev1;
    double *last_ms;      // sde_timing's 4 slots
};

// held by the caller for the whole entry point (calls into one device are
// serialised)
std::mutex &rt_mutex();
// the current device's call context (initialises the device on first use)
int rt_begin(RtCall *c);
// grow-only device scratch slot aux in [0, 4) of the current device
int rt_scratch(int aux, size_t bytes, void **p);
// sets the last-error text and returns code
int rt_fail(int code, const char *msg);

}  // namespace sdegpu
