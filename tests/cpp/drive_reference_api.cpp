// A driver written against the reference's host API names (include/mbcg_lbm.hpp), following
// the reference's main loop (main.cu:25-55): allocate, initialise the jet, then RCS, jet
// boundary conditions and swap per step, with the MLUPS counter and optionally the jet-breakup
// statistics sampler; prints per-field sums and sums of magnitudes.
#include <cstdio>
#include <memory>
#include <vector>

#include "mbcg_lbm.hpp"

int main(int argc, char** argv) {
    const int steps = argc > 1 ? std::atoi(argv[1]) : 20;
    mbcg_params p;
    mbcg_params_default(&p);
    p.nx = 34; p.ny = 30; p.nz = 26;
    p.tau = 0.8; p.sigma = 0.05; p.beta = 0.7; p.jet_radius = 5.0;
    p.jet_center[0] = (p.nx - 1) / 2.0; p.jet_center[1] = (p.nz - 1) / 2.0;
    CudaConfig cfg = make_cudaConfig(p);
    LbmDevice d = allocate_device_memory(cfg);
    launch_InitJet(d.A, cfg);
    MlupsCounter mlups = make_mlups_counter(mlups_active_cells(p));
    // optional jet-breakup statistics (every 5 steps from step 5) into the CSV named by argv[2]
    std::unique_ptr<JetBreakupSampler> sampler;
    if (argc > 2) sampler = std::make_unique<JetBreakupSampler>(argv[2], 5, 5);
    mlups_start(mlups);
    for (int step = 1; step <= steps; ++step) {
        launch_RCS(d.A, d.B, cfg, step);
        launch_JetBoundaryConditions(d.B, d.A, cfg, step);
        swap_moments(d.A, d.B);
        mlups_count_step(mlups);
        if (sampler) {
            MlupsPause pause(mlups); // statistics are not timed, as the reference's output is not
            sampler->sample(step, d.A, cfg);
        }
    }
    mlups_stop(mlups);
    const size_t n = static_cast<size_t>(p.nx) * p.ny * p.nz;
    std::vector<float> h(n);
    real_t* f[MBCG_NFIELDS] = {d.A.rhor, d.A.rhob, d.A.ux, d.A.uy, d.A.uz, d.A.Pixx, d.A.Pixy, d.A.Piyy, d.A.Piyz, d.A.Pizz, d.A.Pixz};
    double sums[MBCG_NFIELDS], abs_sums[MBCG_NFIELDS];
    for (int i = 0; i < MBCG_NFIELDS; ++i) {
        cudaMemcpy(h.data(), f[i], n * sizeof(float), cudaMemcpyDeviceToHost);
        double s = 0.0, a = 0.0;
        for (int z = 1; z < p.nz - 1; ++z)
            for (int y = 0; y < p.ny; ++y)
                for (int x = 1; x < p.nx - 1; ++x) {
                    const double v = h[x + p.nx * (y + static_cast<size_t>(p.ny) * z)];
                    s += v;
                    a += v < 0 ? -v : v;
                }
        sums[i] = s;
        abs_sums[i] = a;
    }
    std::printf("{\"steps\": %d, \"mlups\": %.3f, \"sums\": [", steps, mlups_value(mlups));
    for (int i = 0; i < MBCG_NFIELDS; ++i) std::printf("%s%.17g", i ? ", " : "", sums[i]);
    std::printf("], \"abs_sums\": [");
    for (int i = 0; i < MBCG_NFIELDS; ++i) std::printf("%s%.17g", i ? ", " : "", abs_sums[i]);
    std::printf("]}\n");
    mlups_destroy(mlups);
    free_device_memory(d);
    return 0;
}
