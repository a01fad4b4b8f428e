// The TVAL3 loop (3d/tval3_gpu_3d.cpp:1089-1345) driven from the host over
// device-resident state, in two forms:
//   mode 0: the host enqueues the kernels of one inner iteration and reads the
//           two branch flags (Armijo, inner break) from the control block;
//   mode 1: the whole solve is one CUDA graph.  The loops and branches of the
//           reference (outer while, inner while, first-iteration step size,
//           Armijo failure, restart, multiplier update) are conditional graph
//           nodes whose conditions are set on the device by the epilogues that
//           decide them.  The (at most five) backtracking trials are evaluated
//           in closed form by one kernel (k_bt_coef).  One launch per solve,
//           no host round trip.
// Both forms run the same kernels in the same order, so they give identical
// results.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <typeinfo>
#include <vector>
#include "solver.h"

namespace tv3 {

// A body graph being filled by stream capture.  Between captured sequences,
// conditional nodes are appended with the current tail as dependencies.
struct Body {
    cudaGraph_t g;
    std::vector<cudaGraphNode_t> deps;
    cudaStream_t s;
    bool capturing = false;
    void begin() {
        TV3_CUDA(cudaStreamBeginCaptureToGraph(s, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                               cudaStreamCaptureModeThreadLocal));
        capturing = true;
    }
    void end() {
        cudaStreamCaptureStatus st;
        const cudaGraphNode_t* d = nullptr;
        size_t nd = 0;
        TV3_CUDA(cudaStreamGetCaptureInfo(s, &st, nullptr, nullptr, &d, nullptr, &nd));
        std::vector<cudaGraphNode_t> tail(d, d + nd);
        cudaGraph_t out = g;
        TV3_CUDA(cudaStreamEndCapture(s, &out));
        deps = tail;
        capturing = false;
    }
    // append a conditional node; returns its body graphs
    std::vector<cudaGraph_t> cond(cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type, unsigned size) {
        cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
        np.conditional.handle = h;
        np.conditional.type = type;
        np.conditional.size = size;
        cudaGraphNode_t node;
        TV3_CUDA(cudaGraphAddNode(&node, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &np));
        deps.assign(1, node);
        return std::vector<cudaGraph_t>(np.conditional.phGraph_out, np.conditional.phGraph_out + size);
    }
};


// Elements per block of the vector and reduction kernels, per vector type,
// device and problem shape, as a batch's tuning chose them: a later solver
// of the same shape takes the same grid, so its reductions add in the same
// order as the batch's (results identical to the batched ones).
static std::mutex g_grid_mu;
static std::map<std::string, long> g_grid_epb;

template <class T>
Solver<T>::Solver(const LinOp<T>* A_, int p_, int q_, int r_, const tval3_options& o_, int L_)
    : A(A_), p(p_), q(q_), r(r_), L(std::max(L_, 1)), n((long)p_ * q_ * r_ * std::max(L_, 1)),
      m(A_->m * std::max(L_, 1)), o(o_) {
    if (n >= (1L << 31))
        throw Error{TVAL3_ERR_UNSUPPORTED, "voxels x layers exceeds the 32-bit index range of the stencil kernels"};
    A->prepare(L);
    if (L == 1) {
        PhaseTimer pt(3);
        A->set_volume(p_, q_, r_);
        A->ready();
    }
    const long nvec = 25, mvec = 4;
    nv.alloc(nvec * n);
    mv.alloc(mvec * std::max<long>(m, 1));
    ctl.alloc(1);
    part.alloc(4 * 16384);
    ticket.alloc(1);
    trace.alloc(std::max(1, o.maxit));
    TV3_CUDA(cudaMemset(ticket.p, 0, sizeof(unsigned)));
    TV3_CUDA(cudaMallocHost(&hctl, sizeof(Ctl)));
    T* v = nv.p;
    auto take = [&](long k) { T* t = v; v += k * n; return t; };
    B.p = p; B.q = q; B.r = r; B.L = L; B.n = n; B.m = m;
    B.U[0] = take(1); B.U[1] = take(1);
    B.g[0] = take(1); B.g[1] = take(1);
    B.g2[0] = take(1); B.g2[1] = take(1);
    B.DU[0] = take(3); B.DU[1] = take(3);
    B.d = take(1); B.DtsAtd = take(1); B.Atb = take(1);
    B.W[0] = take(3); B.W[1] = take(3); B.sig = take(3);
    B.rcdU = take(1);
    T* w = mv.p;
    const long mm = std::max<long>(m, 1);
    B.Au[0] = w; B.Au[1] = w + mm; B.b = w + 2 * mm; B.delta = w + 3 * mm;
    B.ctl = ctl.p; B.part = part.p; B.ticket = ticket.p;
    if (o.skipMulRatio != 0.0) {
        last_Au.alloc(std::max<long>(m, 1));
        B.last_Au = last_Au.p;
    }
    // vector/reduction grid: about 1024 elements per block for small problems
    // (so that many small solves can share the GPU), at most eight blocks of
    // 256 threads per SM (a full SM); each launcher trims it further to the
    // blocks its kernel can keep resident.  Partials of the widest reduction
    // (10 values) fit in `part` up to 6,553 blocks.
    set_grid_elems(1024);
    {
        std::lock_guard<std::mutex> lk(g_grid_mu);
        auto it = g_grid_epb.find(grid_key());
        if (it != g_grid_epb.end()) set_grid_elems(it->second);
    }
    B.trace = trace.p;
}

template <class T>
void Solver<T>::set_grid_elems(long epb) {
    const long cap = std::max(1, std::min(num_sms() * 8, 6553));
    B.grid = (int)std::max<long>(1, std::min<long>(cap, (std::max<long>(n, m) + epb - 1) / std::max<long>(epb, 1)));
}

template <class T>
std::string Solver<T>::grid_key() const {
    int dev = 0;
    cudaGetDevice(&dev);
    return std::string(typeid(T).name()) + "/" + std::to_string(dev) + "/" + std::to_string(n) + "/" +
           std::to_string(m);
}

template <class T>
Solver<T>::~Solver() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (rexec) cudaGraphExecDestroy(rexec);
    if (hctl) cudaFreeHost(hctl);
}

template <class T>
MatIO<T> Solver<T>::io_AU() const {
    MatIO<T> io{};
    io.x[0] = B.U[0]; io.x[1] = B.U[1];
    io.y[0] = B.Au[0]; io.y[1] = B.Au[1];
    io.by_parity = 1;
    io.b = B.b; io.delta = B.delta;
    io.ctl = B.ctl; io.part = B.part; io.ticket = B.ticket;
    io.L = L;
    return io;
}
template <class T>
MatIO<T> Solver<T>::io_AtAu() const {
    MatIO<T> io{};
    io.x[0] = B.Au[0]; io.x[1] = B.Au[1];
    io.y[0] = B.g[0]; io.y[1] = B.g[1];
    io.by_parity = 1;
    io.sub = B.Atb;
    io.ctl = B.ctl; io.part = B.part; io.ticket = B.ticket;
    io.L = L;
    return io;
}
template <class T>
MatIO<T> Solver<T>::io_Ad() const {
    MatIO<T> io{};
    io.x[0] = io.x[1] = B.d;
    io.y[0] = io.y[1] = nullptr;
    io.ctl = B.ctl; io.part = B.part; io.ticket = B.ticket;
    io.L = L;
    return io;
}

__global__ void k_init_ctl(Ctl* c, Ctl v) { *c = v; }

// resuming a saved state: the iteration limits of this solver's options, and
// the loop runs again
__global__ void k_resume_ctl(Ctl* c, int maxit, int maxcnt, int pause_at) {
    c->maxit = maxit;
    c->maxcnt = maxcnt;
    c->pause_at = pause_at;
    c->paused = 0;
    c->done = !(c->count_outer < maxcnt && c->count_total < maxit);
    c->err = 0;
    c->launches += 1;
}

template <class T>
void Solver<T>::init_ctl(cudaStream_t s) {
    Ctl c;
    std::memset(&c, 0, sizeof(c));
    c.mu_max = o.mu; c.beta_max = o.beta; c.rate_cnt = o.rate_cnt;
    c.tol = o.tol; c.tol_inn = o.tol_inn; c.c_arm = o.c; c.gamma = o.gamma;
    c.gam0 = o.gam; c.rate_gam = o.rate_gam;
    c.maxcnt = o.maxcnt; c.maxit = o.maxit; c.nonneg = o.nonneg ? 1 : 0; c.iso = (o.tv_type == TVAL3_TV_ISO);
    c.mu = std::min(o.mu0, o.mu);
    c.beta = std::min(o.beta0, o.beta);
    c.muDbeta = c.mu / c.beta;
    c.gam = o.gam;
    c.Q = 1.0;
    c.fst = 1;
    c.scl = 1.0;
    c.pause_at = pause_at > 0 ? pause_at : 0x7fffffff;
    c.skip_ratio = o.skipMulRatio;
    c.max_rel_change = o.maxRelativeChange;
    c.num_init = o.numInitIterations;
    c.launches = 1;  // this kernel
    k_init_ctl<<<1, 1, 0, s>>>(ctl.p, c);
    TV3_CUDA(cudaGetLastError());
}

template <class T>
void Solver<T>::read_ctl(cudaStream_t s) {
    TV3_CUDA(cudaMemcpyAsync(hctl, ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    TV3_CUDA(cudaStreamSynchronize(s));
}

// get_g_gpu (:366-572): Au = A U, g = A^T Au - Atb, g2 = D^T(DU - W), f.
// With the skip-A^T heuristic the A^T product and its alternative (keep the
// previous g) are two IF bodies of the whole-solve graph (body != null), or
// a host branch on the decision in the host-driven form.
template <class T>
void Solver<T>::get_g(int epi, cudaStream_t s, Body* body) {
    A->apply(0, io_AU(), SPMV_LAM35, s);
    if (o.skipMulRatio != 0.0) {
        if (body) {
            // a conditional handle drives one conditional node: fresh pair per call site
            cudaGraphConditionalHandle hm, hk;
            TV3_CUDA(cudaGraphConditionalHandleCreate(&hm, g_top, 1, cudaGraphCondAssignDefault));
            TV3_CUDA(cudaGraphConditionalHandleCreate(&hk, g_top, 0, cudaGraphCondAssignDefault));
            B.h_mult = hm;
            B.h_keep = hk;
        }
        launch_skip_decide<T>(B, epi != EPI_G2_DESCEND, s);
        if (body) {
            body->end();
            {
                Body mb{body->cond(B.h_mult, cudaGraphCondTypeIf, 1)[0], {}, s};
                mb.begin();
                launch_skip_copy<T>(B, 0, s);
                A->apply(1, io_AtAu(), SPMV_SUB, s);
                mb.end();
            }
            {
                Body kb{body->cond(B.h_keep, cudaGraphCondTypeIf, 1)[0], {}, s};
                kb.begin();
                launch_skip_copy<T>(B, 1, s);
                kb.end();
            }
            body->begin();
        } else {
            read_ctl(s);
            if (hctl->do_mult) {
                launch_skip_copy<T>(B, 0, s);
                A->apply(1, io_AtAu(), SPMV_SUB, s);
            } else {
                launch_skip_copy<T>(B, 1, s);
            }
        }
    } else {
        A->apply(1, io_AtAu(), SPMV_SUB, s);
    }
    launch_g2<T>(B, epi, s);
}

// first-iteration step size (:583-611): ||Dd||^2, <d,d>, ||Ad||^2 -> tau
template <class T>
void Solver<T>::tau_first(cudaStream_t s) {
    launch_Dd_norm<T>(B, s);
    A->apply(0, io_Ad(), SPMV_NORM2, s);
}

// start-up (:1115-1149)
template <class T>
void Solver<T>::setup(const void* d_b, cudaStream_t s, Body* body) {
    init_ctl(s);
    if (B.last_Au) TV3_CUDA(cudaMemsetAsync(B.last_Au, 0, std::max<long>(m, 1) * sizeof(T), s));
    TV3_CUDA(cudaMemsetAsync(B.sig, 0, 3 * n * sizeof(T), s));
    TV3_CUDA(cudaMemsetAsync(B.DtsAtd, 0, n * sizeof(T), s));
    if (m > 0) TV3_CUDA(cudaMemsetAsync(B.delta, 0, m * sizeof(T), s));
    launch_scale_b<T>(d_b, B, s);                                    // scaleb_gpu
    MatIO<T> io_atb = plain_io<T>(B.b, B.Atb);
    io_atb.ctl = B.ctl;
    io_atb.L = L;
    A->apply(1, io_atb, SPMV_PLAIN, s);                              // Atb = A^T b
    TV3_CUDA(cudaMemcpyAsync(B.U[0], B.Atb, n * sizeof(T), cudaMemcpyDeviceToDevice, s));   // U = Atb
    TV3_CUDA(cudaMemcpyAsync(B.rcdU, B.Atb, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
    launch_D_only<T>(B, s);
    launch_shrink<T>(B, EPI_G2_INIT, s);
    get_g(EPI_G2_INIT, s, body);
    launch_gradient<T>(B, 0, s);
    TV3_CUDA(cudaGetLastError());
}

template <class T>
void Solver<T>::run_host(cudaStream_t s) {
    if (!(o.maxcnt > 0 && o.maxit > 0)) return;
    read_ctl(s);
    bool fst = hctl->fst != 0;  // 1 after set-up; a resumed state carries its own
    for (;;) {
        // ---- min_u (:823-891); a non-first step size was formed by the
        // previous iteration's gradient kernel
        if (fst) tau_first(s);
        launch_descend<T>(B, 0, s);
        get_g(EPI_G2_DESCEND, s);
        read_ctl(s);
        if (hctl->armijo_fail) {
            // the whole backtracking loop on the closed-form f(alpha), then the
            // accepted point (nothing to apply when all five trials fail)
            launch_bt_coef<T>(B, s);
            launch_bt_apply<T>(B, s);
            read_ctl(s);
            if (hctl->armijo_fail) {  // cnt == 5: exact step from Up
                tau_first(s);
                launch_descend<T>(B, 1, s);
                get_g(EPI_G2_RESTART, s);
            }
            // update_W at the point taken (an accepted full step committed the
            // descent's W in the Armijo kernel instead)
            launch_shrink<T>(B, EPI_G2_UPDATE_W, s);
        }
        // ---- g2 of update_W (:965-1029), gradient, RelChg
        launch_g2_gradient<T>(B, s);
        read_ctl(s);
        fst = false;
        if (hctl->inner_break) {
            launch_outer_relchg<T>(B, s);
            read_ctl(s);
            if (hctl->done) break;
            launch_mlp<T>(B, s);
            launch_outer_grad<T>(B, s);
            read_ctl(s);
            if (hctl->done) break;
            fst = true;
        }
    }
}

// ---------------------------------------------------------------------------
// whole-solve graph
// ---------------------------------------------------------------------------

// Adds the whole solve to `top` as an independent branch (its first nodes are
// roots of `top`), capturing through stream cs.  Several solvers can add
// their branches to one graph; they share nothing on the device.
template <class T>
void Solver<T>::add_to_graph(cudaGraph_t top, const void* d_b, void* d_U, const void* d_Ut, cudaStream_t cs,
                             bool resume) {
    const unsigned run = (o.maxcnt > 0 && o.maxit > 0) ? 1u : 0u;
    // a conditional handle drives one conditional node: the unrolled first
    // inner iteration has its own Armijo and restart handles
    cudaGraphConditionalHandle h_outer, h_inner, h_fst = 0, h_arm, h_restart, h_arm1, h_restart1, h_mlp;
    TV3_CUDA(cudaGraphConditionalHandleCreate(&h_outer, top, run, cudaGraphCondAssignDefault));
    TV3_CUDA(cudaGraphConditionalHandleCreate(&h_inner, top, 1, cudaGraphCondAssignDefault));
    if (resume) TV3_CUDA(cudaGraphConditionalHandleCreate(&h_fst, top, 1, cudaGraphCondAssignDefault));
    TV3_CUDA(cudaGraphConditionalHandleCreate(&h_arm, top, 0, cudaGraphCondAssignDefault));
    TV3_CUDA(cudaGraphConditionalHandleCreate(&h_restart, top, 0, cudaGraphCondAssignDefault));
    if (!resume) {
        TV3_CUDA(cudaGraphConditionalHandleCreate(&h_arm1, top, 0, cudaGraphCondAssignDefault));
        TV3_CUDA(cudaGraphConditionalHandleCreate(&h_restart1, top, 0, cudaGraphCondAssignDefault));
    }
    TV3_CUDA(cudaGraphConditionalHandleCreate(&h_mlp, top, 0, cudaGraphCondAssignDefault));
    g_top = top;
    B.use_graph = 1;
    B.h_inner = h_inner; B.h_mlp = h_mlp;
    // one inner iteration (:1150-1200) appended to body `ib` (not capturing on
    // entry or exit).  first: 0 = no first-step size, 1 = the first-step size
    // unconditionally (the unrolled first iteration of an outer iteration),
    // 2 = an IF node on the control block's fst (a resumed state).
    auto iteration = [&](Body& ib, int first, cudaGraphConditionalHandle harm, cudaGraphConditionalHandle hrs) {
        if (first == 2) {
            ib.begin();
            launch_cond(B.ctl, h_fst, COND_FST, cs);
            ib.end();
            Body t{ib.cond(h_fst, cudaGraphCondTypeIf, 1)[0], {}, cs};
            t.begin();
            tau_first(cs);
            t.end();
        }
        ib.begin();
        if (first == 1) tau_first(cs);
        B.h_arm = harm;
        launch_descend<T>(B, 0, cs);
        get_g(EPI_G2_DESCEND, cs, &ib);  // sets harm
        ib.end();
        {
            Body ab{ib.cond(harm, cudaGraphCondTypeIf, 1)[0], {}, cs};
            ab.begin();
            launch_bt_coef<T>(B, cs);
            launch_bt_apply<T>(B, cs);
            launch_cond(B.ctl, hrs, COND_RESTART, cs);
            ab.end();
            {
                Body rb{ab.cond(hrs, cudaGraphCondTypeIf, 1)[0], {}, cs};
                rb.begin();
                tau_first(cs);
                launch_descend<T>(B, 1, cs);
                get_g(EPI_G2_RESTART, cs, &rb);
                rb.end();
            }
            // update_W at the point taken (an accepted full step committed
            // the descent's W in the Armijo kernel instead)
            ab.begin();
            launch_shrink<T>(B, EPI_G2_UPDATE_W, cs);
            ab.end();
        }
        ib.begin();
        launch_g2_gradient<T>(B, cs);  // sets h_inner
        ib.end();
    };
    try {
        Body tb{top, {}, cs};
        tb.begin();
        if (resume) {
            k_resume_ctl<<<1, 1, 0, cs>>>(B.ctl, o.maxit, o.maxcnt, pause_at > 0 ? pause_at : 0x7fffffff);
            launch_cond(B.ctl, h_outer, COND_NOT_DONE, cs);
        } else {
            setup(d_b, cs, &tb);
        }
        tb.end();
        // outer while
        Body ob{tb.cond(h_outer, cudaGraphCondTypeWhile, 1)[0], {}, cs};
        if (resume) {
            // the resumed state may stop inside an outer iteration: the inner
            // loop starts at once and asks fst on the device
            ob.begin();
            launch_cond(B.ctl, h_inner, COND_ONE, cs);
            ob.end();
            Body ib{ob.cond(h_inner, cudaGraphCondTypeWhile, 1)[0], {}, cs};
            iteration(ib, 2, h_arm, h_restart);
        } else {
            // every outer iteration starts with fst set (start-up, k_mlp): its
            // first inner iteration is unrolled in front of the inner loop, so
            // the loop carries no first-step branch
            iteration(ob, 1, h_arm1, h_restart1);
            Body ib{ob.cond(h_inner, cudaGraphCondTypeWhile, 1)[0], {}, cs};
            iteration(ib, 0, h_arm, h_restart);
        }
        ob.begin();
        launch_outer_relchg<T>(B, cs);  // sets h_mlp
        ob.end();
        {
            Body mb{ob.cond(h_mlp, cudaGraphCondTypeIf, 1)[0], {}, cs};
            mb.begin();
            launch_mlp<T>(B, cs);
            launch_outer_grad<T>(B, cs);
            mb.end();
        }
        ob.begin();
        launch_cond(B.ctl, h_outer, COND_NOT_DONE, cs);
        ob.end();
        tb.begin();
        launch_finalize<T>(B, d_U, d_Ut, cs);
        tb.end();
    } catch (...) {
        B.use_graph = 0;
        throw;
    }
    B.use_graph = 0;
}

template <class T>
void Solver<T>::build_graph(const void* d_b, void* d_U, const void* d_Ut, cudaStream_t s) {
    PhaseTimer pg(4);
    if (gexec) {
        cudaGraphExecDestroy(gexec);
        gexec = nullptr;
    }
    cudaGraph_t top;
    TV3_CUDA(cudaGraphCreate(&top, 0));
    cudaStream_t cs;
    TV3_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    try {
        add_to_graph(top, d_b, d_U, d_Ut, cs);
        TV3_CUDA(cudaGraphInstantiate(&gexec, top, 0));
    } catch (...) {
        cudaStreamDestroy(cs);
        cudaGraphDestroy(top);
        throw;
    }
    cudaStreamDestroy(cs);
    cudaGraphDestroy(top);
    g_b = d_b; g_U = d_U; g_Ut = d_Ut; g_stream = s;
}

template <class T>
void Solver<T>::solve(const void* d_b, void* d_U, const void* d_Ut, tval3_info* info, cudaStream_t s) {
    B.xstar = xstar;
    cudaEvent_t e0, e1;
    TV3_CUDA(cudaEventCreate(&e0));
    TV3_CUDA(cudaEventCreate(&e1));
    TV3_CUDA(cudaEventRecord(e0, s));
    if (mode == 1) {
        if (!gexec || g_b != d_b || g_U != d_U || g_Ut != d_Ut) build_graph(d_b, d_U, d_Ut, s);
        TV3_CUDA(cudaGraphLaunch(gexec, s));
    } else {
        B.use_graph = 0;
        setup(d_b, s);
        run_host(s);
        launch_finalize<T>(B, d_U, d_Ut, s);
    }
    TV3_CUDA(cudaEventRecord(e1, s));
    TV3_CUDA(cudaGetLastError());
    read_ctl(s);
    float ms = 0.f;
    TV3_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    fill_info(info, ms / 1000.0);
}

// ---------------------------------------------------------------------------
// solver state: the control block and every workspace vector, so a solve
// stopped at its iteration limit can be continued later (here or in another
// process) exactly as if it had not stopped
// ---------------------------------------------------------------------------
namespace {
struct StateHeader {
    char magic[8];
    unsigned version, elem_size;
    long long n, m, nv_len, mv_len, last_len;
    int p, q, r, L;
};
}  // namespace

template <class T>
size_t Solver<T>::state_bytes() const {
    return sizeof(StateHeader) + sizeof(Ctl) + (nv.n + mv.n + last_Au.n) * sizeof(T);
}

template <class T>
void Solver<T>::save_state(void* host, cudaStream_t s) {
    StateHeader h{};
    std::memcpy(h.magic, "TVAL3ST", 8);
    h.version = 1;
    h.elem_size = sizeof(T);
    h.n = n; h.m = m; h.nv_len = (long long)nv.n; h.mv_len = (long long)mv.n; h.last_len = (long long)last_Au.n;
    h.p = p; h.q = q; h.r = r; h.L = L;
    char* c = static_cast<char*>(host);
    std::memcpy(c, &h, sizeof(h));
    c += sizeof(h);
    TV3_CUDA(cudaMemcpyAsync(c, ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    c += sizeof(Ctl);
    TV3_CUDA(cudaMemcpyAsync(c, nv.p, nv.n * sizeof(T), cudaMemcpyDeviceToHost, s));
    c += nv.n * sizeof(T);
    if (mv.n) TV3_CUDA(cudaMemcpyAsync(c, mv.p, mv.n * sizeof(T), cudaMemcpyDeviceToHost, s));
    c += mv.n * sizeof(T);
    if (last_Au.n) TV3_CUDA(cudaMemcpyAsync(c, last_Au.p, last_Au.n * sizeof(T), cudaMemcpyDeviceToHost, s));
    TV3_CUDA(cudaStreamSynchronize(s));
}

template <class T>
void Solver<T>::resume(const void* host, void* d_U, const void* d_Ut, tval3_info* info, cudaStream_t s) {
    StateHeader h;
    std::memcpy(&h, host, sizeof(h));
    if (std::memcmp(h.magic, "TVAL3ST", 8) != 0 || h.version != 1)
        throw Error{TVAL3_ERR_ARG, "Argument error: not a solver state!"};
    if (h.elem_size != sizeof(T) || h.n != n || h.m != m || h.nv_len != (long long)nv.n ||
        h.mv_len != (long long)mv.n || h.last_len != (long long)last_Au.n || h.p != p || h.q != q || h.r != r ||
        h.L != L)
        throw Error{TVAL3_ERR_SHAPE, "Argument error: the state belongs to a solver of another shape or type!"};
    const char* c = static_cast<const char*>(host) + sizeof(h);
    TV3_CUDA(cudaMemcpyAsync(ctl.p, c, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    c += sizeof(Ctl);
    TV3_CUDA(cudaMemcpyAsync(nv.p, c, nv.n * sizeof(T), cudaMemcpyHostToDevice, s));
    c += nv.n * sizeof(T);
    if (mv.n) TV3_CUDA(cudaMemcpyAsync(mv.p, c, mv.n * sizeof(T), cudaMemcpyHostToDevice, s));
    c += mv.n * sizeof(T);
    if (last_Au.n) TV3_CUDA(cudaMemcpyAsync(last_Au.p, c, last_Au.n * sizeof(T), cudaMemcpyHostToDevice, s));
    B.xstar = nullptr;
    cudaEvent_t e0, e1;
    TV3_CUDA(cudaEventCreate(&e0));
    TV3_CUDA(cudaEventCreate(&e1));
    TV3_CUDA(cudaEventRecord(e0, s));
    if (mode == 1) {
        if (!rexec || r_U != d_U || r_Ut != d_Ut) {
            if (rexec) cudaGraphExecDestroy(rexec);
            rexec = nullptr;
            cudaGraph_t top;
            TV3_CUDA(cudaGraphCreate(&top, 0));
            cudaStream_t cs;
            TV3_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
            try {
                add_to_graph(top, nullptr, d_U, d_Ut, cs, true);
                TV3_CUDA(cudaGraphInstantiate(&rexec, top, 0));
            } catch (...) {
                cudaStreamDestroy(cs);
                cudaGraphDestroy(top);
                throw;
            }
            cudaStreamDestroy(cs);
            cudaGraphDestroy(top);
            r_U = d_U;
            r_Ut = d_Ut;
        }
        TV3_CUDA(cudaGraphLaunch(rexec, s));
    } else {
        B.use_graph = 0;
        k_resume_ctl<<<1, 1, 0, s>>>(B.ctl, o.maxit, o.maxcnt, pause_at > 0 ? pause_at : 0x7fffffff);
        read_ctl(s);
        if (!hctl->done) run_host(s);
        launch_finalize<T>(B, d_U, d_Ut, s);
    }
    TV3_CUDA(cudaEventRecord(e1, s));
    TV3_CUDA(cudaGetLastError());
    read_ctl(s);
    float ms = 0.f;
    TV3_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    fill_info(info, ms / 1000.0);
}

template <class T>
void Solver<T>::fetch_ctl(cudaStream_t s) {
    TV3_CUDA(cudaMemcpyAsync(hctl, ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
}

template <class T>
void Solver<T>::fill_info(tval3_info* info, double secs) const {
    if (hctl->err) throw Error{TVAL3_ERR_CUDA, "device-side error word set during the solve"};
    if (info) {
        info->total_iters = hctl->count_total;
        info->outer_iters = hctl->count_outer;
        info->rel_chg = hctl->relchgout;
        info->rel_error = hctl->rel_error;
        info->secs = secs;
        info->backtracks = hctl->backtracks;
        info->restarts = hctl->restarts;
        info->final_f = hctl->f;
        info->launches = (int)hctl->launches;
        info->products_T = (o.skipMulRatio != 0.0) ? hctl->products_T : -1;
    }
}

template <class T>
void Solver<T>::read_trace(double* host, int len) {
    int k = std::min(len, (int)trace.n);
    if (k > 0) TV3_CUDA(cudaMemcpy(host, trace.p, k * sizeof(double), cudaMemcpyDeviceToHost));
}

template <class T>
Batch<T>::~Batch() {
    if (gexec) cudaGraphExecDestroy(gexec);
    for (auto* x : s) delete x;
}

template <class T>
cudaGraphExec_t Batch<T>::build(const void* const* b, void* const* U, const void* const* Ut) {
    const size_t k = s.size();
    cudaGraphExec_t ex = nullptr;
    cudaGraph_t top;
    TV3_CUDA(cudaGraphCreate(&top, 0));
    cudaStream_t cs;
    TV3_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    try {
        for (size_t i = 0; i < k; ++i) {
            s[i]->xstar = nullptr;
            s[i]->B.xstar = nullptr;
            s[i]->add_to_graph(top, b[i], U[i], Ut[i], cs);
        }
        TV3_CUDA(cudaGraphInstantiate(&ex, top, 0));
    } catch (...) {
        cudaStreamDestroy(cs);
        cudaGraphDestroy(top);
        throw;
    }
    cudaStreamDestroy(cs);
    cudaGraphDestroy(top);
    return ex;
}

// Tuning of the vector kernels' grid: small slices cannot fill the GPU one
// by one, and how many blocks each slice's kernels take decides how well the
// slices run side by side.  Each candidate runs the whole batch as one graph
// for at most 12 iterations per slice (timed after a warm-up launch); the
// default (1,024 elements per block) is kept unless another is 3 % faster.
// The tuning solves write the caller's U, which the real solve overwrites.
template <class T>
void Batch<T>::tune(const void* const* b, void* const* U, const void* const* Ut, cudaStream_t st) {
    const size_t k = s.size();
    const long cand[] = {1024, 512, 2048, 4096};
    std::vector<int> keep(k);
    for (size_t i = 0; i < k; ++i) {
        keep[i] = s[i]->o.maxit;
        s[i]->o.maxit = std::min(s[i]->o.maxit, 12);
    }
    cudaEvent_t e0, e1;
    TV3_CUDA(cudaEventCreate(&e0));
    TV3_CUDA(cudaEventCreate(&e1));
    float best = 0.f;
    long best_c = 1024;
    try {
        for (long c : cand) {
            for (auto* x : s) x->set_grid_elems(c);
            cudaGraphExec_t ex = build(b, U, Ut);
            TV3_CUDA(cudaGraphLaunch(ex, st));
            TV3_CUDA(cudaEventRecord(e0, st));
            TV3_CUDA(cudaGraphLaunch(ex, st));
            TV3_CUDA(cudaEventRecord(e1, st));
            TV3_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            TV3_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            cudaGraphExecDestroy(ex);
            if (c == 1024 || ms < 0.97f * best) {
                best = ms;
                best_c = c;
            }
        }
    } catch (...) {
        for (size_t i = 0; i < k; ++i) s[i]->o.maxit = keep[i];
        for (auto* x : s) x->set_grid_elems(1024);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (size_t i = 0; i < k; ++i) s[i]->o.maxit = keep[i];
    grid_elems = best_c;
    std::lock_guard<std::mutex> lk(g_grid_mu);
    for (auto* x : s) {
        x->set_grid_elems(best_c);
        g_grid_epb[x->grid_key()] = best_c;
    }
}

template <class T>
void Batch<T>::solve(const void* const* b, void* const* U, const void* const* Ut, tval3_info* infos,
                     cudaStream_t st) {
    const size_t k = s.size();
    bool same = gexec && g_b.size() == k;
    for (size_t i = 0; same && i < k; ++i) same = g_b[i] == b[i] && g_U[i] == U[i] && g_Ut[i] == Ut[i];
    if (!same) {
        if (gexec) {
            cudaGraphExecDestroy(gexec);
            gexec = nullptr;
        }
        if (!tuned) {
            tuned = true;
            if (k > 1) tune(b, U, Ut, st);
        }
        gexec = build(b, U, Ut);
        g_b.assign(b, b + k);
        g_U.assign(U, U + k);
        g_Ut.assign(Ut, Ut + k);
    }
    cudaEvent_t e0, e1;
    TV3_CUDA(cudaEventCreate(&e0));
    TV3_CUDA(cudaEventCreate(&e1));
    TV3_CUDA(cudaEventRecord(e0, st));
    TV3_CUDA(cudaGraphLaunch(gexec, st));
    TV3_CUDA(cudaEventRecord(e1, st));
    for (auto* x : s) x->fetch_ctl(st);
    TV3_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    TV3_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (size_t i = 0; i < k; ++i) s[i]->fill_info(infos ? infos + i : nullptr, ms / 1000.0);
}

template struct Solver<float>;
template struct Solver<double>;
template struct Solver<df64>;
template struct Batch<float>;
template struct Batch<double>;
template struct Batch<df64>;

}  // namespace tv3
