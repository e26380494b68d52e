// A program written against the drop-in C++ API, as a user of the
// reference's classes would write it (CSRHost, ArnoldiParams,
// TimeSteppingParams, ArnoldiRunner): it loads a .bincsr matrix, sets the
// ArnoldiParams and, optionally, edits the runner's public ts_params before
// the solve, runs compute_expmv and writes y. The GPU tests compile it with
// g++ against include/matrix_exp_krylov.hpp and compare its [STEP] lines and
// y with the reference's own output for the same settings.
//
//   runner_check matrix.bincsr v.bin y.bin m t tol max_restarts
//                [dt_init dt_min dt_max tol_step max_steps max_rejects
//                 safety grow shrink adapt_m m_max m_step]
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <vector>

#include "matrix_exp_krylov.hpp"

int main(int argc, char** argv) {
    if (argc != 8 && argc != 20) {
        std::cerr << "usage: runner_check matrix.bincsr v.bin y.bin m t tol max_restarts [12 ts_params]" << std::endl;
        return 2;
    }
    CSRHost A;
    A.from_binary_csr(argv[1]);
    std::vector<double> v(static_cast<size_t>(A.rows));
    {
        std::ifstream f(argv[2], std::ios::binary);
        if (!f.read(reinterpret_cast<char*>(v.data()), sizeof(double) * v.size())) {
            std::cerr << "cannot read " << argv[2] << std::endl;
            return 2;
        }
    }
    ArnoldiParams params(std::atoi(argv[4]), std::atof(argv[5]), std::atof(argv[6]), std::atoi(argv[7]), true);
    ArnoldiRunner runner(1, params, A.rows, A.cols, A.nnz);
    if (argc == 20) {
        TimeSteppingParams& ts = runner.ts_params;
        ts.dt_init = std::atof(argv[8]);
        ts.dt_min = std::atof(argv[9]);
        ts.dt_max = std::atof(argv[10]);
        ts.tol_step = std::atof(argv[11]);
        ts.max_steps = std::atoi(argv[12]);
        ts.max_rejects = std::atoi(argv[13]);
        ts.safety = std::atof(argv[14]);
        ts.grow = std::atof(argv[15]);
        ts.shrink = std::atof(argv[16]);
        ts.adapt_m = std::atoi(argv[17]) != 0;
        ts.m_max = std::atoi(argv[18]);
        ts.m_step = std::atoi(argv[19]);
    }
    std::vector<CSRHost> parts = A.partition_rows(1);
    std::vector<CSRHost::GhostMap> maps(1);
    runner.init_all_devices(parts, {0}, maps);
    std::vector<double> y(static_cast<size_t>(A.rows), 0.0);
    runner.compute_expmv(v, y);
    std::ofstream out(argv[3], std::ios::binary);
    out.write(reinterpret_cast<const char*>(y.data()), sizeof(double) * y.size());
    std::cout << "RESULT restarts_done=" << runner.restarts_done << " converged=" << (runner.converged ? 1 : 0)
              << std::endl;
    runner.destroy();
    return 0;
}
