// Owning device buffer (cudaMalloc / cudaFree), move-only.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include "ops.h"

namespace tv3 {

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
            void* q = nullptr;
            TV3_CUDA(cudaMalloc(&q, n_ * sizeof(T)));
            p = static_cast<T*>(q);
            n = n_;
        }
    }
    void view(T* q, size_t n_) {
        release();
        p = q;
        n = n_;
        own = false;
    }
    void release() {
        if (p && own) cudaFree(p);
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
// stream-ordered allocation on the legacy stream from the device's default
// memory pool, which keeps up to 4 GB of freed memory for the next request,
// so the temporaries of an operator build cost no driver mapping after the
// first build.  Only for buffers used by work on the legacy stream (or on
// streams that synchronise with it) and freed in the same scope.
void tmp_pool_init();
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
