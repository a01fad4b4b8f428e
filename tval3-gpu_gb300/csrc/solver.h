// TVAL3 solver workspace and loop driver (internal).
#pragma once

#include <string>
#include <vector>
#include "dbuf.h"
#include "ops.h"
#include "tval3/tval3_c.h"

namespace tv3 {

struct Body;  // a graph body being filled by stream capture (solver.cu)

template <class T>
struct Solver {
    const LinOp<T>* A;
    int p, q, r;
    int L;         // layers sharing A (the 2D entry's b.len / A.rows)
    long n, m;     // vector lengths (voxels * L, rays * L)
    tval3_options o;
    DBuf<T> nv, mv;
    DBuf<Ctl> ctl;
    DBuf<double> part;
    DBuf<unsigned> ticket;
    DBuf<double> trace;
    DBuf<T> last_Au;      // skip-A^T heuristic only
    Ctl* hctl = nullptr;  // pinned mirror of the control block
    SolverBufs<T> B{};
    int mode = 0;         // 0: host-driven loop, 1: CUDA graph with conditional nodes
    int pause_at = 0;     // > 0: stop after this many total iterations, resumable
    const void* xstar = nullptr;  // caller-type reference solution for the error trace
    // graph of the whole solve (mode 1), rebuilt when its inputs change
    cudaGraphExec_t gexec = nullptr;
    const void* g_b = nullptr;
    void* g_U = nullptr;
    const void* g_Ut = nullptr;
    cudaStream_t g_stream = nullptr;
    cudaGraph_t g_top = nullptr;  // the graph being built by add_to_graph
    cudaGraphExec_t rexec = nullptr;  // resume graph (mode 1)
    void* r_U = nullptr;
    const void* r_Ut = nullptr;

    Solver(const LinOp<T>* A_, int p_, int q_, int r_, const tval3_options& o_, int L_ = 1);
    // grid of the vector and reduction kernels: about epb elements per block
    // (1,024 by default, or the value a batch's tuning stored for this shape)
    void set_grid_elems(long epb);
    std::string grid_key() const;
    ~Solver();
    // b, U and Ut are device arrays of the caller-facing type Ext<T>
    // (float for float vectors, double for double and double-float vectors)
    void solve(const void* d_b, void* d_U, const void* d_Ut, tval3_info* info, cudaStream_t s);
    void read_trace(double* host, int len);
    // the whole solve as an independent branch of `top` (mode 1 form); with
    // resume, the loop continues from the current state instead of set-up
    void add_to_graph(cudaGraph_t top, const void* d_b, void* d_U, const void* d_Ut, cudaStream_t cs,
                      bool resume = false);
    // solver state (control block and workspace) to host memory and back
    size_t state_bytes() const;
    void save_state(void* host, cudaStream_t s);
    void resume(const void* host, void* d_U, const void* d_Ut, tval3_info* info, cudaStream_t s);
    // enqueue the copy of the control block to its pinned mirror; after the
    // stream is synchronised, fill_info reports it
    void fetch_ctl(cudaStream_t s);
    void fill_info(tval3_info* info, double secs) const;

   private:
    void init_ctl(cudaStream_t s);
    void read_ctl(cudaStream_t s);
    void setup(const void* d_b, cudaStream_t s, Body* body = nullptr);
    void get_g(int epi, cudaStream_t s, Body* body = nullptr);
    void tau_first(cudaStream_t s);
    void run_host(cudaStream_t s);
    void build_graph(const void* d_b, void* d_U, const void* d_Ut, cudaStream_t s);
    MatIO<T> io_AU() const;
    MatIO<T> io_AtAu() const;
    MatIO<T> io_Ad() const;
};

// Many independent solves (e.g. the slices of a 2D stack) as ONE CUDA graph:
// every solver's whole-solve graph is a parallel branch, each with its own
// conditional loops, so slices that converge early simply stop while the
// others go on, and small slices fill the GPU together.
template <class T>
struct Batch {
    std::vector<Solver<T>*> s;  // owned
    cudaGraphExec_t gexec = nullptr;
    std::vector<const void*> g_b, g_Ut;
    std::vector<void*> g_U;
    bool tuned = false;
    long grid_elems = 1024;  // the tuned elements per block of the vector kernels

    ~Batch();
    // b[i], U[i], Ut[i] (may be NULL): device arrays of the type Ext<T>;
    // infos[i].secs is the time of the whole batch
    void solve(const void* const* b, void* const* U, const void* const* Ut, tval3_info* infos, cudaStream_t st);

   private:
    cudaGraphExec_t build(const void* const* b, void* const* U, const void* const* Ut);
    // times short solves of the whole batch with 512 ... 4,096 elements per
    // block of the vector kernels and keeps the fastest
    void tune(const void* const* b, void* const* U, const void* const* Ut, cudaStream_t st);
};

}  // namespace tv3
