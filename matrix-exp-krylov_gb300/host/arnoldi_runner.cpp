// DeviceContext and ArnoldiRunner on top of the mexk C ABI.
//
// Mirrors the reference classes (kol-di/matrix-exp-krylov main.cu:747-1125
// and 1253-2081) for one device. compute_expmv hands the whole solve to
// mexk_expmv, then prints the attempt log in the reference's [STEP] format,
// the [FLOPs] model (main.cu:1539-1565) and the METRIC line.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <vector>

#include <dlfcn.h>

#include <fstream>
#include <string>

#include "matrix_exp_krylov.hpp"

namespace {

// A trained controller network: $<env>, else the file the package ships
// next to the build directory (../mexk/<file>). An empty vector when the
// file is optional and absent; a missing required file exits as the
// reference does on a bad input.
std::vector<float> load_controller_net(const char* env_name = "MEXK_CONTROLLER_NET",
                                       const char* file = "controller_net.f32", bool required = true) {
    std::string path;
    if (const char* env = std::getenv(env_name); env && env[0]) {
        path = env;
    } else {
        Dl_info info;
        if (dladdr(reinterpret_cast<void*>(&load_controller_net), &info) && info.dli_fname) {
            std::string lib(info.dli_fname);
            path = lib.substr(0, lib.find_last_of('/')) + "/../mexk/" + file;
        }
    }
    std::ifstream f(path, std::ios::binary);
    std::vector<float> w(MEXK_NET_TOTAL);
    if (!f || !f.read(reinterpret_cast<char*>(w.data()), sizeof(float) * w.size())) {
        if (!required) return {};
        std::cerr << "Error: could not read the controller network from " << path << std::endl;
        std::exit(EXIT_FAILURE);
    }
    return w;
}

[[noreturn]] void die(const char* what, int rc) {
    std::cerr << "mexk Error: " << what << ": " << mexk_error_string(rc);
    const char* d = mexk_last_error_detail();
    if (d && d[0]) std::cerr << " (" << d << ")";
    std::cerr << std::endl;
    std::exit(EXIT_FAILURE);
}

}  // namespace

void DeviceContext::init_handles() {}

void DeviceContext::create_streams() {
    if (handle) return;
    int rc = mexk_context_create(device_id, &handle);
    if (rc != MEXK_OK) die("mexk_context_create", rc);
}

void DeviceContext::alloc_from(const CSRHost& part, int global_cols, int m_alloc_max) {
    (void)global_cols;
    if (!handle) create_streams();
    local_rows = part.rows;
    local_nnz = static_cast<int>(part.nnz);
    std::cout << "GPU " << device_id << " allocating: local_rows=" << local_rows << ", local_nnz=" << local_nnz
              << std::endl;
    allocated_m_max = std::max(1, m_alloc_max);
    int rc = mexk_context_upload_csr(handle, part.rows, part.nnz, part.row_ptr.data(), part.col_idx.data(),
                                     part.values.data(), allocated_m_max);
    if (rc != MEXK_OK) die("mexk_context_upload_csr", rc);
}

void DeviceContext::create_descriptors(const CSRHost&, int, const CSRHost::GhostMap&, int, int) {}

void DeviceContext::destroy() {
    if (handle) mexk_context_destroy(handle);
    handle = nullptr;
}

ArnoldiRunner::ArnoldiRunner(int n_gpus, const ArnoldiParams& arnoldi_params, int total_rows, int total_cols,
                             long long total_nnz)
    : num_gpus(n_gpus), params(arnoldi_params), global_rows(total_rows), global_cols(total_cols),
      global_nnz(total_nnz) {
    device_contexts.reserve(static_cast<size_t>(std::max(1, num_gpus)));
    for (int i = 0; i < std::max(1, num_gpus); ++i) device_contexts.emplace_back(i);
    // Derived time-stepping parameters (main.cu:1292-1305); the device
    // controller computes the same values from ArnoldiParams.
    ts_params.dt_max = params.t;
    ts_params.dt_min = std::max(1e-12, params.t * 1e-6);
    const double denom = (params.max_restarts > 0) ? params.max_restarts : 1;
    ts_params.dt_init = params.t / denom;
    ts_params.tol_step = params.tol;
    ts_params.max_steps = (params.max_restarts > 0) ? params.max_restarts : 1000;
    ts_params.max_rejects = 20;
    ts_params.safety = 0.8;
    ts_params.grow = 1.5;
    ts_params.shrink = 0.5;
    ts_params.adapt_m = false;
    ts_params.m_max = params.m;
    ts_params.m_step = 0;
}

namespace {

// The checks init_all_devices makes before any allocation (main.cu:1308-1330).
void check_runner_shape(const ArnoldiParams& params, int global_rows, int global_cols) {
    if (params.m >= global_rows) {
        std::cerr << "ERROR: Requested Arnoldi m=" << params.m << " must be less than global_rows=" << global_rows
                  << std::endl;
        std::exit(EXIT_FAILURE);
    }
    if (global_rows != global_cols) {
        std::cerr << "ERROR: Matrix must be square. rows=" << global_rows << " cols=" << global_cols << std::endl;
        std::exit(EXIT_FAILURE);
    }
    if (params.m > MEXK_M_MAX) {
        std::cerr << "ERROR: Requested Arnoldi m=" << params.m << " exceeds the supported maximum " << MEXK_M_MAX
                  << std::endl;
        std::exit(EXIT_FAILURE);
    }
}

// Krylov dimension the device allocation must hold (main.cu:1343).
int alloc_dimension(const ArnoldiParams& params, const TimeSteppingParams& ts, int global_rows) {
    int m = std::max(params.m, ts.m_max > 0 ? ts.m_max : params.m);
    // the basis needs m < n; a larger m_max is refused when a solve asks for it
    m = std::min(m, std::max(params.m, global_rows - 1));
    return std::min(m, MEXK_M_MAX);
}

}  // namespace

void ArnoldiRunner::init_from_context(mexk_context_t ctx, int device_id) {
    check_runner_shape(params, global_rows, global_cols);
    DeviceContext& dc = device_contexts[0];
    dc.device_id = device_id;
    dc.handle = ctx;
    dc.local_rows = global_rows;
    dc.local_nnz = static_cast<int>(global_nnz);
    dc.allocated_m_max = alloc_dimension(params, ts_params, global_rows);
    std::cout << "GPU " << dc.device_id << " allocating: local_rows=" << dc.local_rows
              << ", local_nnz=" << dc.local_nnz << std::endl;
}

void ArnoldiRunner::init_all_devices(const std::vector<CSRHost>& partitions, const std::vector<int>& device_ids,
                                     const std::vector<CSRHost::GhostMap>& ghost_maps_in) {
    ghost_maps = ghost_maps_in;
    if (static_cast<int>(device_ids.size()) != num_gpus) {
        std::cerr << "ERROR: device_ids size (" << device_ids.size() << ") must match num_gpus (" << num_gpus << ")"
                  << std::endl;
        std::exit(EXIT_FAILURE);
    }
    check_runner_shape(params, global_rows, global_cols);
    // Row partitions hold global column indices: stacking them restores A.
    CSRHost full;
    full.rows = 0;
    full.cols = global_cols;
    full.row_ptr.assign(1, 0);
    for (const CSRHost& p : partitions) {
        const int base = full.row_ptr.back();
        for (int r = 0; r < p.rows; ++r) full.row_ptr.push_back(base + p.row_ptr[r + 1]);
        full.col_idx.insert(full.col_idx.end(), p.col_idx.begin(), p.col_idx.begin() + p.nnz);
        full.values.insert(full.values.end(), p.values.begin(), p.values.begin() + p.nnz);
        full.rows += p.rows;
    }
    full.nnz = static_cast<long long>(full.col_idx.size());
    DeviceContext& dc = device_contexts[0];
    dc.device_id = device_ids.empty() ? 0 : device_ids[0];
    if (partitions.size() > 1)
        std::cerr << "[mexk] warning: " << partitions.size() << " row partitions are concatenated onto GPU "
                  << dc.device_id << "; this build solves on one device" << std::endl;
    dc.init_handles();
    dc.create_streams();
    const int alloc_m = alloc_dimension(params, ts_params, global_rows);
    dc.alloc_from(full, global_cols, alloc_m);
    dc.create_descriptors(full, global_cols, CSRHost::GhostMap(), 0, alloc_m);
}

void ArnoldiRunner::compute_expmv(const std::vector<double>& v_host, std::vector<double>& y_host) {
    const auto t0 = std::chrono::steady_clock::now();
    if (mode != ExpmvMode::AdaptiveTimeStepping) {
        std::cerr << "Expmv mode not implemented" << std::endl;
        return;
    }
    DeviceContext& dc = device_contexts[0];
    mexk_params_t p;
    p.m = params.m;
    p.t = params.t;
    p.tol = params.tol;
    p.max_restarts = params.max_restarts;
    p.reorthogonalize = params.reorthogonalize ? 1 : 0;
    p.precision = precision;
    p.controller = controller;
    p.ortho_window = ortho_window;
    // The caller's time-stepping parameters, read on every solve as the
    // reference's compute_expmv does (main.cu:1426, 1476-1516).
    mexk_stepping_t ts;
    ts.dt_init = ts_params.dt_init;
    ts.dt_min = ts_params.dt_min;
    ts.dt_max = ts_params.dt_max;
    ts.tol_step = ts_params.tol_step;
    ts.max_steps = ts_params.max_steps;
    ts.max_rejects = ts_params.max_rejects;
    ts.safety = ts_params.safety;
    ts.grow = ts_params.grow;
    ts.shrink = ts_params.shrink;
    ts.adapt_m = ts_params.adapt_m ? 1 : 0;
    ts.m_max = ts_params.m_max;
    ts.m_step = ts_params.m_step;
    p.stepping = &ts;
    if (ts.adapt_m && ts.m_step > 0 && ts.m_max > params.m && ts.m_max > dc.allocated_m_max) {
        // main.cu:1441-1444
        std::cerr << "ERROR: m_current exceeds allocated_m_max on GPU 0" << std::endl;
        std::exit(EXIT_FAILURE);
    }
    if (controller == MEXK_CTRL_LEARNED && !net_loaded) {
        const std::vector<float> w = load_controller_net();
        int lrc = mexk_context_set_controller(dc.handle, w.data(), static_cast<int>(w.size()));
        if (lrc != MEXK_OK) die("mexk_context_set_controller", lrc);
        // the network priced for window-2 cycles, when shipped
        const std::vector<float> ww =
            load_controller_net("MEXK_CONTROLLER_NET_WINDOW", "controller_net_window.f32", false);
        if (!ww.empty()) {
            lrc = mexk_context_set_window_controller(dc.handle, ww.data(), static_cast<int>(ww.size()));
            if (lrc != MEXK_OK) die("mexk_context_set_window_controller", lrc);
        }
        net_loaded = true;
    }
    int rc = mexk_expmv(dc.handle, &p, v_host.data(), y_host.data(), &last_result);
    if (rc != MEXK_OK) die("mexk_expmv", rc);
    converged = last_result.converged != 0;
    restarts_done = last_result.restarts_done;
    last_residual = last_result.last_residual;
    int count = 0;
    mexk_get_steps(dc.handle, nullptr, 0, &count);
    last_steps.resize(static_cast<size_t>(count));
    if (count > 0) mexk_get_steps(dc.handle, last_steps.data(), count, &count);
    if (verbose) {
        for (const mexk_step_t& s : last_steps) {
            if (log_h_columns)
                for (int j = 0; j < s.m_used; ++j)
                    std::cout << "    H_m column " << j << " stored. Current H_m size: " << (s.m_basis + 1) << "x"
                              << s.m_basis << std::endl;
            std::cout << "[STEP] t=" << s.t_done << " dt=" << s.dt << " err=" << s.err << " m_used=" << s.m_used
                      << " accepts=" << s.accepts << " rejects=" << s.rejects << std::endl;
        }
        // An abort (20 rejects) is the only way to finish unconverged at t_done = t.
        if (!converged && last_result.t_done >= params.t && params.t > 0)
            std::cerr << "[STEP] rejected too many times, aborting" << std::endl;
        const double N = static_cast<double>(global_rows);
        const double nnz = static_cast<double>(global_nnz);
        const double m = static_cast<double>(params.m);
        const double S = static_cast<double>(restarts_done);
        const double seg = 2.0 * nnz * m + 4.0 * N * m * (m + 1.0) + 5.0 * N * m + 2.0 * N;
        const double gpu_total = 3.0 * N * S + S * seg;
        const double cpu_seg = 2.0 * 1.0 * m * m * m + 2.0 * m * m;
        std::cout << "[FLOPs] N=" << N << " nnz=" << nnz << " m=" << m << " steps=" << S << std::endl;
        std::cout << "[FLOPs] GPU segment: " << seg << " | GPU total: " << gpu_total << std::endl;
        std::cout << "[FLOPs] CPU segment: " << cpu_seg << " | CPU total: " << S * cpu_seg << " (C_exp=" << 1.0 << ")"
                  << std::endl;
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        std::cout << "METRIC total_compute_expmv_ms=" << ms << std::endl;
    }
}

void ArnoldiRunner::destroy() {
    for (DeviceContext& dc : device_contexts) dc.destroy();
}
