// Written the way a caller of the 2D reference is (2d/tval3_gpu.h,
// 2d/container_host.h): untemplated mat_host / sparse_mat_host, the sparse
// matrix in one format (CSC by default), tval3_gpu(U, A, b, opts) with the
// defaulted Ut and pagelocked arguments, and the dense overload.  On a GPU
// host it reconstructs a tiny image three ways and prints the counts.
#include <cstdio>
#include <vector>

#include "tval3/tval3_2d.hpp"

int main() {
    // 2 x 2 image (4 pixels), 4 rays: rays 0, 1 see pixels 0 and 3; rays 2, 3
    // see pixel pairs (0, 1) and (2, 3).  CSC arrays: column c's rows.
    std::vector<int> cptr = {0, 2, 3, 4, 6}, cind = {0, 2, 2, 3, 1, 3};
    std::vector<float> cval = {1, 1, 1, 1, 1, 1};
    sparse_mat_host A(4, 4, 6, cval.data(), cptr.data(), cind.data());
    mat_host U(2, 2), b(4);
    b[0] = 1.f; b[1] = 2.f; b[2] = 1.5f; b[3] = 3.f;
    tval3_options opts;
    opts.maxit = 20;
    try {
        const tval3_info info = tval3_gpu(U, A, b, opts);
        std::printf("sparse iters %d outer %d U0 %.4f\n", info.total_iters, info.outer_iters, U[0]);
        // the same matrix dense (column-major rows x cols)
        mat_host Ad(4, 4);
        for (int c = 0; c < 4; ++c)
            for (int k = cptr[c]; k < cptr[c + 1]; ++k) Ad[cind[k] + 4 * c] = cval[k];
        mat_host U2(2, 2), Ut(4);
        for (int i = 0; i < 4; ++i) Ut[i] = U[i];
        const tval3_info info2 = tval3_gpu(U2, Ad, b, opts, Ut, true);
        std::printf("dense iters %d rel_error %.3e\n", info2.total_iters, info2.rel_error);
        // the CSR of the same matrix, built from the CSC arrays
        std::vector<int> rind(6), cnt(5, 0);
        std::vector<float> rval(6);
        for (int c = 0; c < 4; ++c)
            for (int k = cptr[c]; k < cptr[c + 1]; ++k) ++cnt[cind[k] + 1];
        for (int r = 0; r < 4; ++r) cnt[r + 1] += cnt[r];
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (int c = 0; c < 4; ++c)
            for (int k = cptr[c]; k < cptr[c + 1]; ++k) {
                rind[fill[cind[k]]] = c;
                rval[fill[cind[k]]++] = cval[k];
            }
        sparse_mat_host Ar(4, 4, 6, rval.data(), cnt.data(), rind.data(), sparse_mat_csr);
        mat_host U3(2, 2);
        const tval3_info info3 = tval3_gpu(U3, Ar, b, opts);
        float d = 0.f;
        for (int i = 0; i < 4; ++i) d += (U3[i] - U[i]) * (U3[i] - U[i]);
        std::printf("csr iters %d same %d\n", info3.total_iters, d == 0.f ? 1 : 0);
    } catch (const tval3_gpu_exception& e) {
        std::printf("tval3_gpu_exception: %s\n", e.what());
        return 2;
    }
    // copies and assignment as in the reference
    mat_host V(U);
    try {
        mat_host W(3, 3);
        W = V;
        return 4;
    } catch (const illegal_mat_gpu_assignment&) {
        std::printf("assignment rejected\n");
    }
    mat_host bad(5);
    try {
        tval3_gpu(U, A, bad, opts);
        return 3;
    } catch (const tval3_gpu_exception& e) {
        std::printf("rejected: %s\n", e.what());
    }
    return 0;
}
