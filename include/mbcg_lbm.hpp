// mbcg_lbm.hpp -- the reference solver's host API, re-expressed over the mbcg C ABI.
//
// A program written against the reference's headers (memory.cuh, launch.cuh,
// utilities/mlups_count.cuh, io/vtiWriter.cuh) keeps its names and call order:
//
//     MomentsDevice, LbmDevice, LbmHost           memory.cuh:14-50
//     allocate_device_memory / free_device_memory memory.cuh:153-194
//     allocate_host_memory / free_host_memory     memory.cuh:135-186
//     launch_InitJet / launch_InitStaticBubble / launch_InitRTI      launch.cuh:14-72
//     launch_RCS / launch_JetBoundaryConditions   launch.cuh:78-94
//     swap_moments, copy_out_D2H                  memory.cuh:200-217
//     MlupsCounter, make_mlups_counter, mlups_*   utilities/mlups_count.cuh:14-216
//     write_vti_step_device                       io/vtiWriter.cuh:151-164
//
// Differences, all forced by moving compile-time constants to run time: the lattice size and
// physics come from an mbcg_params carried in CudaConfig; errors throw mbcg::Error instead of
// exit(1) (utilities/cudaUtilities.cuh:9-19); launch_RCS etc. take the time-step index so the
// seeded inlet noise is reproducible.  Arrays use the reference's dense layout (pitch = nx).
#ifndef MBCG_LBM_HPP
#define MBCG_LBM_HPP

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>

#include "mbcg.h"

namespace mbcg {

struct Error : std::runtime_error {
    explicit Error(const std::string& what) : std::runtime_error(what) {}
};

inline void check(int rc, const char* what) {
    if (rc != MBCG_OK) throw Error(std::string(what) + ": " + mbcg_last_error());
}
inline void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw Error(std::string(what) + ": " + cudaGetErrorString(e));
}

} // namespace mbcg

using real_t = float;
using label_t = uint32_t;

// memory.cuh:14-29
struct MomentsDevice {
    real_t* rhor = nullptr;
    real_t* rhob = nullptr;
    real_t* ux = nullptr;
    real_t* uy = nullptr;
    real_t* uz = nullptr;
    real_t* Pixx = nullptr;
    real_t* Pixy = nullptr;
    real_t* Piyy = nullptr;
    real_t* Piyz = nullptr;
    real_t* Pizz = nullptr;
    real_t* Pixz = nullptr;
};

struct LbmDevice {
    MomentsDevice A; // current state
    MomentsDevice B; // next state
};

struct LbmHost {
    real_t* rhor = nullptr;
    real_t* rhob = nullptr;
    real_t* ux = nullptr;
    real_t* uy = nullptr;
    real_t* uz = nullptr;
};

// utilities/cudaConfig.cuh:28-43, carrying the run-time case parameters
struct CudaConfig {
    mbcg_params params{};
    cudaStream_t stream = nullptr;
};

inline CudaConfig make_cudaConfig(const mbcg_params& p, cudaStream_t s = nullptr) {
    CudaConfig c;
    c.params = p;
    c.stream = s;
    return c;
}

inline size_t bytes_cell(const mbcg_params& p) {
    return static_cast<size_t>(p.nx) * p.ny * p.nz * sizeof(real_t);
}

inline mbcg_moments to_view(const MomentsDevice& m, const mbcg_params& p) {
    mbcg_moments v{};
    real_t* const f[MBCG_NFIELDS] = {m.rhor, m.rhob, m.ux, m.uy, m.uz, m.Pixx, m.Pixy, m.Piyy, m.Piyz, m.Pizz, m.Pixz};
    for (int i = 0; i < MBCG_NFIELDS; ++i) v.f[i] = f[i];
    v.pitch = p.nx;
    v.precision = MBCG_FP32;
    return v;
}

// memory.cuh:153-164: both states, zeroed
inline LbmDevice allocate_device_memory(const CudaConfig& cfg) {
    LbmDevice d{};
    const size_t b = bytes_cell(cfg.params);
    for (MomentsDevice* m : {&d.A, &d.B}) {
        real_t** f[MBCG_NFIELDS] = {&m->rhor, &m->rhob, &m->ux, &m->uy, &m->uz, &m->Pixx,
                                    &m->Pixy, &m->Piyy, &m->Piyz, &m->Pizz, &m->Pixz};
        for (auto* pp : f) {
            mbcg::check_cuda(cudaMalloc(reinterpret_cast<void**>(pp), b), "cudaMalloc");
            mbcg::check_cuda(cudaMemset(*pp, 0, b), "cudaMemset");
        }
    }
    return d;
}

inline void free_device_memory(LbmDevice& d) {
    for (MomentsDevice* m : {&d.A, &d.B}) {
        real_t* f[MBCG_NFIELDS] = {m->rhor, m->rhob, m->ux, m->uy, m->uz, m->Pixx, m->Pixy, m->Piyy, m->Piyz, m->Pizz, m->Pixz};
        for (real_t* p : f)
            if (p) cudaFree(p);
        *m = MomentsDevice{};
    }
}

inline LbmHost allocate_host_memory(const CudaConfig& cfg) {
    LbmHost h{};
    const size_t b = bytes_cell(cfg.params);
    for (real_t** p : {&h.rhor, &h.rhob, &h.ux, &h.uy, &h.uz})
        mbcg::check_cuda(cudaMallocHost(reinterpret_cast<void**>(p), b), "cudaMallocHost");
    return h;
}

inline void free_host_memory(LbmHost& h) {
    for (real_t* p : {h.rhor, h.rhob, h.ux, h.uy, h.uz})
        if (p) cudaFreeHost(p);
    h = LbmHost{};
}

// launch.cuh:14-72: initial conditions (the jet also applies its initial boundary pass)
inline void launch_Init(MomentsDevice A, const CudaConfig& cfg, int ic) {
    mbcg_params p = cfg.params;
    p.ic = ic;
    const mbcg_moments v = to_view(A, p);
    mbcg::check(mbcg_init_moments(&p, &v, reinterpret_cast<mbcg_stream_t>(cfg.stream)), "launch_Init");
    mbcg::check_cuda(cudaStreamSynchronize(cfg.stream), "launch_Init");
}
inline void launch_InitJet(MomentsDevice A, const CudaConfig& cfg) { launch_Init(A, cfg, MBCG_IC_JET); }
inline void launch_InitStaticBubble(MomentsDevice A, const CudaConfig& cfg) { launch_Init(A, cfg, MBCG_IC_BUBBLE); }
inline void launch_InitRTI(MomentsDevice A, const CudaConfig& cfg) { launch_Init(A, cfg, MBCG_IC_RTI); }

// launch.cuh:89-94 -> the fused sm_103a kernel without its boundary pass
inline void launch_RCS(const MomentsDevice A, MomentsDevice B, const CudaConfig& cfg, int64_t step) {
    const mbcg_moments a = to_view(A, cfg.params), b = to_view(B, cfg.params);
    mbcg::check(mbcg_rcs_moments(&cfg.params, &a, &b, step, reinterpret_cast<mbcg_stream_t>(cfg.stream)),
                "launch_RCS");
}

// launch.cuh:78-83
inline void launch_JetBoundaryConditions(MomentsDevice B, const MomentsDevice Aold, const CudaConfig& cfg,
                                         int64_t step) {
    const mbcg_moments b = to_view(B, cfg.params), a = to_view(Aold, cfg.params);
    mbcg::check(mbcg_bc_moments(&cfg.params, &b, &a, step, reinterpret_cast<mbcg_stream_t>(cfg.stream)),
                "launch_JetBoundaryConditions");
}

// memory.cuh:200-203
inline void swap_moments(MomentsDevice& A, MomentsDevice& B) noexcept { std::swap(A, B); }

// memory.cuh:209-217
inline void copy_out_D2H(LbmHost& h, const MomentsDevice& d, const CudaConfig& cfg) {
    const size_t b = bytes_cell(cfg.params);
    const std::pair<real_t*, const real_t*> f[] = {{h.rhor, d.rhor}, {h.rhob, d.rhob}, {h.ux, d.ux}, {h.uy, d.uy}, {h.uz, d.uz}};
    for (const auto& c : f) mbcg::check_cuda(cudaMemcpy(c.first, c.second, b, cudaMemcpyDeviceToHost), "copy_out_D2H");
}

// ------------------------------------------------------------------ MLUPS counter
// utilities/mlups_count.cuh:14-216: same surface and definition (cells x steps / s / 1e6 over
// the (nx-2)(ny-2)(nz-2) active cells, cudaEvent timing with pause / resume).
struct MlupsCounter {
    std::uint64_t cells_per_step = 0;
    std::uint64_t steps = 0;
    float elapsed_ms = 0.0f;
    cudaEvent_t start_event = nullptr;
    cudaEvent_t stop_event = nullptr;
    bool running = false;
};

inline std::uint64_t mlups_active_cells(const mbcg_params& p) {
    return static_cast<std::uint64_t>(mbcg_active_nodes(&p));
}
inline MlupsCounter make_mlups_counter(std::uint64_t cells_per_step) {
    MlupsCounter c{};
    c.cells_per_step = cells_per_step;
    mbcg::check_cuda(cudaEventCreate(&c.start_event), "cudaEventCreate");
    mbcg::check_cuda(cudaEventCreate(&c.stop_event), "cudaEventCreate");
    return c;
}
inline void mlups_start(MlupsCounter& c) {
    c.steps = 0;
    c.elapsed_ms = 0.0f;
    mbcg::check_cuda(cudaEventRecord(c.start_event), "cudaEventRecord");
    c.running = true;
}
inline void mlups_pause(MlupsCounter& c) {
    if (!c.running) return;
    mbcg::check_cuda(cudaEventRecord(c.stop_event), "cudaEventRecord");
    mbcg::check_cuda(cudaEventSynchronize(c.stop_event), "cudaEventSynchronize");
    float ms = 0.0f;
    mbcg::check_cuda(cudaEventElapsedTime(&ms, c.start_event, c.stop_event), "cudaEventElapsedTime");
    c.elapsed_ms += ms;
    c.running = false;
}
inline void mlups_resume(MlupsCounter& c) {
    if (c.running) return;
    mbcg::check_cuda(cudaEventRecord(c.start_event), "cudaEventRecord");
    c.running = true;
}
inline void mlups_stop(MlupsCounter& c) { mlups_pause(c); }
inline void mlups_destroy(MlupsCounter& c) {
    if (c.start_event) cudaEventDestroy(c.start_event);
    if (c.stop_event) cudaEventDestroy(c.stop_event);
    c.start_event = c.stop_event = nullptr;
}
inline void mlups_count_step(MlupsCounter& c, std::uint64_t n = 1) noexcept { c.steps += n; }
inline double mlups_elapsed_seconds(MlupsCounter& c) {
    float ms = c.elapsed_ms;
    if (c.running) {
        mbcg::check_cuda(cudaEventRecord(c.stop_event), "cudaEventRecord");
        mbcg::check_cuda(cudaEventSynchronize(c.stop_event), "cudaEventSynchronize");
        float w = 0.0f;
        mbcg::check_cuda(cudaEventElapsedTime(&w, c.start_event, c.stop_event), "cudaEventElapsedTime");
        ms += w;
    }
    return static_cast<double>(ms) * 1.0e-3;
}
inline std::uint64_t mlups_lattice_updates(const MlupsCounter& c) noexcept { return c.cells_per_step * c.steps; }
inline double mlups_value(MlupsCounter& c) {
    const double s = mlups_elapsed_seconds(c);
    return s <= 0.0 ? 0.0 : static_cast<double>(mlups_lattice_updates(c)) / (s * 1.0e6);
}
inline void mlups_print(MlupsCounter& c, std::ostream& out = std::cout) {
    const auto flags = out.flags();
    const auto prec = out.precision();
    out << std::fixed << std::setprecision(3) << "MLUPS: " << mlups_value(c) << " | elapsed: " << mlups_elapsed_seconds(c)
        << " s | steps: " << c.steps << " | cells/step: " << c.cells_per_step << '\n';
    out.flags(flags);
    out.precision(prec);
}
struct MlupsPause {
    explicit MlupsPause(MlupsCounter& c) : counter(c), was_running(c.running) { mlups_pause(counter); }
    ~MlupsPause() {
        if (was_running) mlups_resume(counter);
    }
    MlupsPause(const MlupsPause&) = delete;
    MlupsPause& operator=(const MlupsPause&) = delete;

private:
    MlupsCounter& counter;
    bool was_running;
};

// ------------------------------------------------------------------ VTI output
// io/vtiWriter.cuh:60-164: the five fields rhor, rhob, ux, uy, uz over the full extent
// (ghosts included), ASCII VTK ImageData.
inline void write_vti(const std::filesystem::path& filename, const LbmHost& h, const mbcg_params& p) {
    if (!filename.parent_path().empty()) std::filesystem::create_directories(filename.parent_path());
    std::ofstream out(filename);
    if (!out) throw mbcg::Error("Cannot open VTI file for writing: " + filename.string());
    out << "<?xml version=\"1.0\"?>\n<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
    out << "  <ImageData WholeExtent=\"0 " << p.nx - 1 << " 0 " << p.ny - 1 << " 0 " << p.nz - 1
        << "\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n";
    out << "    <Piece Extent=\"0 " << p.nx - 1 << " 0 " << p.ny - 1 << " 0 " << p.nz - 1 << "\">\n";
    out << "      <PointData Scalars=\"rhor\">\n";
    const std::pair<const char*, const real_t*> fields[] = {{"rhor", h.rhor}, {"rhob", h.rhob}, {"ux", h.ux}, {"uy", h.uy}, {"uz", h.uz}};
    for (const auto& f : fields) {
        out << "        <DataArray type=\"Float32\" Name=\"" << f.first << "\" format=\"ascii\">\n";
        out << std::scientific << std::setprecision(8);
        const size_t nx = p.nx, nxy = static_cast<size_t>(p.nx) * p.ny;
        for (int z = 0; z < p.nz; ++z) {
            for (int y = 0; y < p.ny; ++y) {
                for (int x = 0; x < p.nx; ++x) out << static_cast<float>(f.second[x + y * nx + z * nxy]) << " ";
                out << "\n";
            }
        }
        out << "        </DataArray>\n";
    }
    out << "      </PointData>\n      <CellData>\n      </CellData>\n    </Piece>\n  </ImageData>\n</VTKFile>\n";
    if (!out) throw mbcg::Error("Error while finalizing VTI file: " + filename.string());
}

inline std::filesystem::path vti_filename(int step, const std::filesystem::path& folder) {
    std::ostringstream name;
    name << "jet_" << std::setw(8) << std::setfill('0') << step << ".vti";
    return folder / name.str();
}

inline void write_vti_step_device(int step, const MomentsDevice& d, LbmHost& h, const CudaConfig& cfg,
                                  const std::filesystem::path& folder) {
    mbcg::check_cuda(cudaDeviceSynchronize(), "write_vti_step_device");
    copy_out_D2H(h, d, cfg);
    write_vti(vti_filename(step, folder), h, cfg.params);
}

// ------------------------------------------------------------------ jet-breakup statistics
// The reference declares a statistics sampler's interval and start (NSTATS_SAMPLE = 20,
// stats_start_tstar = 7000: constants.cuh:11,53) but implements none.  This one records the
// in-situ phase statistics (mbcg_phase_statistics_moments, connected regions included) of a
// state every `every` steps from step `start` on, one CSV row per sample: the jet's penetration,
// its number of regions, the detached droplets and their volume, the largest region, the
// interface area and node count, and the injected phase's volume.
class JetBreakupSampler {
  public:
    JetBreakupSampler(const std::filesystem::path& csv, int every = 20, long long start = 7000)
        : every_(every > 0 ? every : 1), start_(start) {
        if (!csv.parent_path().empty()) std::filesystem::create_directories(csv.parent_path());
        out_.open(csv);
        if (!out_) throw mbcg::Error("Cannot open statistics file: " + csv.string());
        out_ << "step,penetration,regions,detached,detached_volume,largest_region,interface_area,"
                "interface_nodes,injected_volume\n";
    }
    // samples the state if step is due; returns whether it did
    bool sample(long long step, const MomentsDevice& A, const CudaConfig& cfg) {
        if (step < start_ || (step - start_) % every_ != 0) return false;
        const mbcg_moments m = to_view(A, cfg.params);
        mbcg_phase_stats st;
        mbcg::check(mbcg_phase_statistics_moments(&cfg.params, &m, MBCG_STATS_COMPONENTS, &st,
                                                  reinterpret_cast<mbcg_stream_t>(cfg.stream)),
                    "phase statistics");
        out_ << step << ',' << st.penetration << ',' << st.components << ',' << st.detached << ','
             << st.detached_volume << ',' << st.largest_component << ',' << std::setprecision(10)
             << st.interface_area << ',' << st.interface_nodes << ',' << st.volume_tracked << '\n';
        out_.flush();
        return true;
    }

  private:
    int every_;
    long long start_;
    std::ofstream out_;
};

#endif // MBCG_LBM_HPP
