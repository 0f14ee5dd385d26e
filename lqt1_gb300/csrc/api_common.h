// api_common.h -- helpers shared by the host API translation units.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/lqt.h"
#include "lqt_internal.h"

namespace lqt {

extern thread_local std::string g_err;
int fail(int code, const std::string &msg);

// CUDA call inside an entry point returning an lqt status.
#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return ::lqt::fail(LQT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
    } while (0)

// Owns device allocations of a handle; everything is freed on destruction.
struct DevMem {
    std::vector<void *> ptrs;
    int alloc(void **p, size_t bytes)
    {
        *p = nullptr;
        if (bytes == 0) bytes = 16;
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            *p = nullptr;
            g_err = std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e);
            return LQT_ERR_NOMEM;
        }
        ptrs.push_back(*p);
        return LQT_OK;
    }
    void reset()
    {
        for (void *p : ptrs) cudaFree(p);
        ptrs.clear();
    }
    ~DevMem() { reset(); }
};

void initial_state(double v0, double *s);
ModelK make_modelk(const lqt_model &m);
StepK make_stepk(double dt);
int check_model(const lqt_model &m);
void time_axis(double dt, double t_stop, std::vector<double> &times);
void stim_windows(const std::vector<double> &times, int64_t nsteps, double dt, double bcl, double start, double dur,
                  int beats, std::vector<Win> &out);
int64_t pad128(int64_t n);

template <typename R> int batch_max_ctas_per_sm(int threads, int minb);
template <typename R> std::vector<std::pair<int, int>> batch_variants();

}  // namespace lqt
