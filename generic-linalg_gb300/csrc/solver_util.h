// solver_util.h -- host-side plumbing shared by the solvers: scratch allocation on the
// library stream, host/device staging of phi/phi0, the CUDA-graph while-loop that drives an
// iteration body without host round trips, timing, and the reference's verbosity output.
#pragma once

#include <string>
#include <vector>

#include "operator.h"

namespace glinalg {

// Stream-ordered scratch allocations released when the object goes out of scope.
class Scratch {
  public:
    explicit Scratch(cudaStream_t st) : st_(st) {}
    ~Scratch()
    {
        for (void *p : ptrs_) cudaFreeAsync(p, st_);
    }
    template <class T>
    glinalg_status alloc(T **out, size_t count)
    {
        void *p = nullptr;
        cudaError_t e = lib_malloc_async(&p, sizeof(T) * (count ? count : 1), st_);
        if (e != cudaSuccess) {
            set_last_error(std::string("stream-ordered allocation: ") + cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? GLINALG_ERROR_OUT_OF_MEMORY : GLINALG_ERROR_CUDA;
        }
        ptrs_.push_back(p);
        *out = (T *)p;
        return GLINALG_SUCCESS;
    }
    template <class T>
    glinalg_status zeros(T **out, size_t count)
    {
        GL_TRY(alloc(out, count));
        GL_CUDA(cudaMemsetAsync(*out, 0, sizeof(T) * (count ? count : 1), st_));
        return GLINALG_SUCCESS;
    }

  private:
    cudaStream_t st_;
    std::vector<void *> ptrs_;
};

// Whether solver loops run as CUDA graphs with conditional WHILE nodes (the default) or from
// a host loop that launches the same kernels and reads the stop flag after every pass
// (environment GLINALG_SOLVER_GRAPHS=0; used for per-kernel profiling, since profilers do not
// resolve kernel nodes inside conditional graphs, and as a fallback).
bool use_graphs();

// Ends the enclosing while loop once *done is set (one thread).
__global__ void k_loop_guard(const int *done, cudaGraphConditionalHandle h);

// Runs `body(stream)` (the kernels of one iteration, each returning early once *done is set)
// until *done: as one CUDA graph with a conditional WHILE node whose body is captured from
// `body` followed by k_loop_guard, or from a host loop.  Returns once the work is enqueued
// (graph) or finished (host loop).
template <class F>
glinalg_status run_loop(cudaStream_t st, const int *done, F body)
{
    if (!use_graphs()) {
        for (long pass = 0;; pass++) {
            GL_TRY(body(st));
            int h = 0;
            GL_CUDA(cudaMemcpyAsync(&h, done, sizeof(int), cudaMemcpyDeviceToHost, st));
            GL_CUDA(cudaStreamSynchronize(st));
            if (h) return GLINALG_SUCCESS;
        }
    }
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ex = nullptr;
    cudaGraphConditionalHandle h = 0;
    glinalg_status s = GLINALG_SUCCESS;
    auto fail = [&](cudaError_t e, const char *what) {
        set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
        s = GLINALG_ERROR_CUDA;
    };
    cudaError_t e;
    do {
        if ((e = cudaGraphCreate(&g, 0)) != cudaSuccess) { fail(e, "cudaGraphCreate"); break; }
        if ((e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) { fail(e, "cudaGraphConditionalHandleCreate"); break; }
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        if ((e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np)) != cudaSuccess) { fail(e, "cudaGraphAddNode"); break; }
        cudaGraph_t bg = np.conditional.phGraph_out[0];
        // capture on a private stream; the graph is launched on `st`
        cudaStream_t cs = capture_stream();
        if ((e = cudaStreamBeginCaptureToGraph(cs, bg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) { fail(e, "capture"); break; }
        glinalg_status bs = body(cs);
        if (bs == GLINALG_SUCCESS) k_loop_guard<<<1, 32, 0, cs>>>(done, h);
        cudaGraph_t captured = nullptr;
        e = cudaStreamEndCapture(cs, &captured);
        if (bs != GLINALG_SUCCESS) { s = bs; break; }
        if (e != cudaSuccess) { fail(e, "end capture"); break; }
        if ((e = cudaGraphInstantiate(&ex, g, 0)) != cudaSuccess) { fail(e, "cudaGraphInstantiate"); break; }
        if ((e = cudaGraphLaunch(ex, st)) != cudaSuccess) { fail(e, "cudaGraphLaunch"); break; }
    } while (0);
    // the executable graph may be destroyed while its launch is in flight
    if (ex) cudaGraphExecDestroy(ex);
    if (g) cudaGraphDestroy(g);
    return s;
}

// Device copies of phi (in/out) and phi0 (in) for a solve; copies back on finish().
struct Staged {
    double2 *x = nullptr;
    const double2 *b = nullptr;
    glinalg_status stage(Scratch &sc, double *phi, const double *phi0, long n, bool dev,
                         cudaStream_t st);
    glinalg_status finish(double *phi, long n, bool dev, cudaStream_t st);
};

struct EventTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    EventTimer();
    ~EventTimer();
    void start(cudaStream_t st) { cudaEventRecord(a, st); }
    void stop(cudaStream_t st) { cudaEventRecord(b, st); }
    double ms();
};

// generic BLAS launchers (device pointers, results into device slots)
glinalg_status launch_norm2(const double2 *a, long n, double *partials, unsigned *counter,
                            double *out, cudaStream_t st);
glinalg_status launch_dot(const double2 *a, const double2 *b, long n, double *partials,
                          unsigned *counter, double2 *out, cudaStream_t st);
glinalg_status launch_diffnorm2(const double2 *a, const double2 *b, long n, double *partials,
                                unsigned *counter, double *out, cudaStream_t st);
glinalg_status launch_sub(double2 *out, const double2 *a, const double2 *b, long n,
                          cudaStream_t st);  // out = a - b

// The reference's verbosity output (verbosity.h:73-131), byte-compatible lines on stdout.
struct Verb {
    int level = 0;
    std::string prefix;
    int precond_level = 0;
    std::string precond_prefix;
    bool present = false;
    static Verb from(const glinalg_verbosity *v);
    Verb restart_inner() const;  // shuffle_verbosity_restart (verbosity.h:27-43)
    Verb precond_inner() const;  // shuffle_verbosity_precond (verbosity.h:46-67)
    void resid(const std::string &alg, int iter, int ops, double relres) const;
    void summary(const std::string &alg, bool success, int iter, int ops, double relres) const;
    // whether summary() prints (a caller can skip the work of its arguments otherwise)
    bool prints_summary() const { return present && (level == 1 || level == 2 || level == 3); }
    void summary_multi(bool success, int iter, int ops, const double *relres, int n) const;
    void restart(const std::string &alg, int iter, int ops, double relres) const;
};

void fill_name(glinalg_info *info, const std::string &name);

// Validates the common solver arguments and returns whether pointers are device pointers.
glinalg_status check_solver_args(glinalg_operator op, const void *phi, const void *phi0,
                                 int size, bool *dev, const glinalg_solver_params *params);

}  // namespace glinalg
