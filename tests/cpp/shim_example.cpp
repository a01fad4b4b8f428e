// Compiles against include/tval3/tval3.hpp the way reference callers are
// written (tval3_gpu_3d(U, A, b, opts, Ut, ...)) and, when run on a GPU host,
// reconstructs a tiny problem and prints the iteration count.
#include <cstdio>
#include <vector>

#include "tval3/tval3.hpp"

int main() {
    // 2 x 2 image, 4 rays: rows 0,1 see single pixels, rows 2,3 see pairs
    std::vector<int> ptr = {0, 1, 2, 4, 6}, ind = {0, 3, 0, 1, 2, 3};
    std::vector<float> val = {1, 1, 1, 1, 1, 1};
    sparse_mat_host<float> A(4, 4, 6, val.data(), ptr.data(), ind.data(), nullptr, nullptr, nullptr);
    mat_host<float> U(2, 2, 1), b(4), Ut(0);
    b[0] = 1.f; b[1] = 2.f; b[2] = 1.5f; b[3] = 3.f;
    tval3_options<float> opts;
    opts.maxit = 20;
    try {
        tval3_info<float> info = tval3_gpu_3d(U, A, b, opts, Ut, true);
        std::printf("iters %d outer %d U0 %.4f\n", info.total_iters, info.outer_iters, U[0]);
    } catch (const tval3_gpu_exception& e) {
        std::printf("tval3_gpu_exception: %s\n", e.what());
        return 2;
    }
    // argument errors are rethrown as tval3_gpu_exception
    mat_host<float> bad(5);
    try {
        tval3_gpu_3d(U, A, bad, opts, Ut, true);
        return 3;
    } catch (const tval3_gpu_exception& e) {
        std::printf("rejected: %s\n", e.what());
    }
    return 0;
}
