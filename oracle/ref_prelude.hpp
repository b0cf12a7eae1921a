// ref_prelude.hpp -- force-included before the reference's headers when they are compiled
// as host C++ for the parity shim (oracle/ref_shim.cpp).  TEST INFRASTRUCTURE ONLY.
//
// The reference keeps every parameter as a compile-time constant in constants.cuh and
// real_t in utilities/types.cuh.  This prelude defines both include guards and supplies the
// same names with the values of one test configuration (passed as -DREF_* macros), using
// the reference's own definitions for every derived constant (constants.cuh:55-93) so the
// arithmetic matches the reference exactly.  It also empties the CUDA execution-space
// keywords so the device functions compile for the host.
#pragma once
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#ifndef __CUDACC__
#undef __host__
#undef __device__
#undef __global__
#undef __forceinline__
#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#endif

#ifndef REF_REAL
#define REF_REAL float
#endif

#define TYPES_CUH
using real_t = REF_REAL;
using label_t = uint32_t;

#define CONSTANTS_CUH
inline constexpr int NSTEP = 1;
inline constexpr int NOUTPUT = 0;
inline constexpr int NSTATS_SAMPLE = 20;
inline constexpr label_t NX = static_cast<label_t>(REF_NX);
inline constexpr label_t NZ = static_cast<label_t>(REF_NZ);
inline constexpr label_t NY = static_cast<label_t>(REF_NY);
inline constexpr label_t NXNY = NX * NY;
inline constexpr label_t Ncells = NX * NY * NZ;
#if defined(LBM_D3Q19)
inline constexpr label_t Q = 19;
#else
inline constexpr label_t Q = 27;
#endif
inline constexpr std::size_t bytesCell = std::size_t(Ncells) * sizeof(real_t);
inline constexpr real_t jet_radius = static_cast<real_t>(REF_JET_RADIUS);
inline constexpr real_t jet_x0 = static_cast<real_t>(NX - 1) / static_cast<real_t>(2);
inline constexpr real_t jet_z0 = static_cast<real_t>(NZ - 1) / static_cast<real_t>(2);
inline constexpr real_t jet_velocity = static_cast<real_t>(REF_JET_VELOCITY);
inline constexpr real_t bubble_radius = static_cast<real_t>(REF_BUBBLE_RADIUS);
inline constexpr real_t bubble_x0 = static_cast<real_t>(NX - 1) / static_cast<real_t>(2);
inline constexpr real_t bubble_y0 = static_cast<real_t>(NY - 1) / static_cast<real_t>(2);
inline constexpr real_t bubble_z0 = static_cast<real_t>(NZ - 1) / static_cast<real_t>(2);
inline constexpr real_t pi = static_cast<real_t>(3.141592653589793);
inline constexpr real_t rti_y0 = static_cast<real_t>(NY - 1) / static_cast<real_t>(2);
inline constexpr real_t rti_amplitude = static_cast<real_t>(REF_RTI_AMPLITUDE);
inline constexpr real_t gravity = static_cast<real_t>(1.0e-6);
inline constexpr real_t rti_interface_width = static_cast<real_t>(REF_RTI_WIDTH);
inline constexpr int rti_mode_x = 1;
inline constexpr int rti_mode_z = 1;
inline constexpr real_t stats_start_tstar = static_cast<real_t>(7000.0);
inline constexpr real_t cs2 = static_cast<real_t>(1.0 / 3.0);
inline constexpr real_t cs4 = cs2 * cs2;
inline constexpr real_t cs6 = cs4 * cs2;
inline constexpr real_t inv_cs2 = static_cast<real_t>(1) / cs2;
inline constexpr real_t inv_cs4 = static_cast<real_t>(1) / cs4;
inline constexpr real_t inv_cs6 = static_cast<real_t>(1) / cs6;
inline constexpr real_t inv_2cs2 = static_cast<real_t>(1) / (static_cast<real_t>(2) * cs2);
inline constexpr real_t inv_2cs4 = static_cast<real_t>(1) / (static_cast<real_t>(2) * cs4);
inline constexpr real_t inv_6cs6 = static_cast<real_t>(1.0) / (static_cast<real_t>(6.0) * cs6);
inline constexpr real_t inv_2cs6 = static_cast<real_t>(1.0) / (static_cast<real_t>(2.0) * cs6);
inline constexpr real_t half = static_cast<real_t>(0.5);
inline constexpr real_t rhor0 = static_cast<real_t>(1);
inline constexpr real_t rhob0 = static_cast<real_t>(1);
inline constexpr real_t Re = static_cast<real_t>(100);
inline constexpr real_t nu = (static_cast<real_t>(2) * jet_radius * jet_velocity) / Re;
inline constexpr real_t taur = static_cast<real_t>(REF_TAU);
inline constexpr real_t taub = static_cast<real_t>(REF_TAU);
inline constexpr real_t omegar = static_cast<real_t>(1) / taur;
inline constexpr real_t omegab = static_cast<real_t>(1) / taub;
inline constexpr real_t oms = static_cast<real_t>(1) - omegab;
inline constexpr real_t We = static_cast<real_t>(2500);
inline constexpr real_t sigma = static_cast<real_t>(REF_SIGMA);
inline constexpr real_t beta_recolor = static_cast<real_t>(REF_BETA);
inline constexpr real_t sigma_over_4cs4 = sigma / (static_cast<real_t>(4) * cs4);
