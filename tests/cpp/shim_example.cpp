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
    // double geometry overloads (3d/tval3_gpu_3d.cpp:58-69): a 4 x 4 x 1
    // volume, 2 emitters x 2 receivers, Siddon rays between voxel centres
    int xe[2] = {0, 3}, ye[2] = {0, 0}, ze[2] = {0, 0}, xr[2] = {3, 0}, yr[2] = {3, 3}, zr[2] = {0, 0};
    geometry_host G;
    G.num_emitters = 2; G.num_receivers = 2;
    G.x_emitters = xe; G.y_emitters = ye; G.z_emitters = ze;
    G.x_receivers = xr; G.y_receivers = yr; G.z_receivers = zr;
    G.rv_x = 4; G.rv_y = 4; G.rv_z = 1;
    G.traversal = TVAL3_TRAVERSAL_SIDDON;
    mat_host<double> Ud(4, 4, 1), bd(4), Utd(0);
    for (int i = 0; i < 4; ++i) bd[i] = 1.0 + i;
    tval3_options<double> od;
    od.maxit = 10;
    std::vector<int> gptr = {0, 1, 2, 3, 4}, gind = {0, 5, 10, 15};
    std::vector<double> gval = {1, 1, 1, 1};
    sparse_mat_host<double> Ag(4, 16, 4, gval.data(), gptr.data(), gind.data(), nullptr, nullptr, nullptr);
    try {
        tval3_info<double> ig = tval3_gpu_3d(Ud, G, bd, od, Utd, true);
        tval3_info<double> igs = tval3_gpu_3d(Ud, G, Ag, bd, od, Utd, true);
        std::printf("geometry f64 iters %d, geometry+sparse f64 iters %d\n", ig.total_iters, igs.total_iters);
    } catch (const tval3_gpu_exception& e) {
        std::printf("tval3_gpu_exception: %s\n", e.what());
        return 4;
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
