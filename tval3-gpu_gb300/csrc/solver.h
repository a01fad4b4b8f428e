// TVAL3 solver workspace and loop driver (internal).
#pragma once

#include "dbuf.h"
#include "ops.h"
#include "tval3/tval3_c.h"

namespace tv3 {

template <class T>
struct Solver {
    const LinOp<T>* A;
    int p, q, r;
    long n, m;
    tval3_options o;
    DBuf<T> nv, mv;
    DBuf<Ctl> ctl;
    DBuf<double> part;
    DBuf<unsigned> ticket;
    DBuf<double> trace;
    Ctl* hctl = nullptr;  // pinned mirror of the control block
    SolverBufs<T> B{};
    int mode = 0;         // 0: host-driven loop, 1: CUDA graph with conditional nodes
    const void* xstar = nullptr;  // caller-type reference solution for the error trace
    // graph of the whole solve (mode 1), rebuilt when its inputs change
    cudaGraphExec_t gexec = nullptr;
    const void* g_b = nullptr;
    void* g_U = nullptr;
    const void* g_Ut = nullptr;
    cudaStream_t g_stream = nullptr;

    Solver(const LinOp<T>* A_, int p_, int q_, int r_, const tval3_options& o_);
    ~Solver();
    // b, U and Ut are device arrays of the caller-facing type Ext<T>
    // (float for float vectors, double for double and double-float vectors)
    void solve(const void* d_b, void* d_U, const void* d_Ut, tval3_info* info, cudaStream_t s);
    void read_trace(double* host, int len);

   private:
    void init_ctl(cudaStream_t s);
    void read_ctl(cudaStream_t s);
    void setup(const void* d_b, cudaStream_t s);
    void get_g(int epi, cudaStream_t s);
    void tau_first(cudaStream_t s);
    void run_host(cudaStream_t s);
    void build_graph(const void* d_b, void* d_U, const void* d_Ut, cudaStream_t s);
    MatIO<T> io_AU() const;
    MatIO<T> io_AtAu() const;
    MatIO<T> io_Ad() const;
};

}  // namespace tv3
