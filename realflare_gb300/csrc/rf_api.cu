// rf_api.cu — library identification and the per-thread text of the last CUDA error.
#include <stdio.h>
#include <string.h>

#include "rf_common.cuh"

#include <atomic>

namespace rf {
namespace {
thread_local char g_last_error[256] = "";
std::atomic<long long> g_launches{0};
}  // namespace
void set_error_text(const char* text) { snprintf(g_last_error, sizeof g_last_error, "%s", text); }
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void set_cuda_error(cudaError_t e) {
    const char* name = cudaGetErrorName(e);
    const char* text = cudaGetErrorString(e);
    snprintf(g_last_error, sizeof g_last_error, "%s: %s", name ? name : "?", text ? text : "?");
}
}  // namespace rf

extern "C" const char* rf_version(void) { return "realflare_gb300 0.1.0 (sm_103a)"; }
extern "C" const char* rf_last_cuda_error(void) { return rf::g_last_error; }
extern "C" long long rf_launch_count(void) { return rf::g_launches.load(std::memory_order_relaxed); }
