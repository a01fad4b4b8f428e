// Owning device buffer, move-only.  Memory comes from the device's default
// stream-ordered pool (see tmp_pool_init: freed memory is kept for the next
// request, so repeated operator and solver set-ups cost no driver mapping).
// It keeps cudaMalloc/cudaFree's guarantees: an allocation is complete before
// alloc() returns (usable from any stream), and release() waits for the
// device before handing the memory back to the pool.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include "ops.h"

namespace tv3 {

void tmp_pool_init();

// bytes of DBuf memory allocated and not yet released by the calling thread
// (the operator entry points report their creation's growth of it)
inline thread_local long long dbuf_live_bytes = 0;

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    bool own = true;  // false: a view of another buffer (never freed here)
    DBuf() {}
    explicit DBuf(size_t n_) { alloc(n_); }
    void alloc(size_t n_) {
        release();
        if (n_) {
            tmp_pool_init();
            void* q = nullptr;
            TV3_CUDA(cudaMallocAsync(&q, n_ * sizeof(T), 0));
            TV3_CUDA(cudaStreamSynchronize(0));
            p = static_cast<T*>(q);
            n = n_;
            dbuf_live_bytes += (long long)(n_ * sizeof(T));
        }
    }
    void view(T* q, size_t n_) {
        release();
        p = q;
        n = n_;
        own = false;
    }
    void release() {
        if (p && own) {
            cudaDeviceSynchronize();
            cudaFreeAsync(p, 0);
            dbuf_live_bytes -= (long long)(n * sizeof(T));
        }
        p = nullptr;
        n = 0;
        own = true;
    }
    ~DBuf() { release(); }
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), own(o.own) {
        o.p = nullptr;
        o.n = 0;
    }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            own = o.own;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
};

// Scratch buffer of a build step (sort keys, index maps, cub workspace):
// stream-ordered allocation and free on the legacy stream, with no device
// synchronisation.  Only for buffers used by work on the legacy stream (or on
// streams that synchronise with it) and freed in the same scope.
template <class T>
struct TmpBuf {
    T* p = nullptr;
    size_t n = 0;
    TmpBuf() {}
    explicit TmpBuf(size_t n_) { alloc(n_); }
    void alloc(size_t n_) {
        release();
        if (n_) {
            tmp_pool_init();
            void* q = nullptr;
            TV3_CUDA(cudaMallocAsync(&q, n_ * sizeof(T), 0));
            p = static_cast<T*>(q);
            n = n_;
        }
    }
    void release() {
        if (p) cudaFreeAsync(p, 0);
        p = nullptr;
        n = 0;
    }
    ~TmpBuf() { release(); }
    TmpBuf(const TmpBuf&) = delete;
    TmpBuf& operator=(const TmpBuf&) = delete;
};

}  // namespace tv3
