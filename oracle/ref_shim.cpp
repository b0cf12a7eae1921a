// ref_shim.cpp -- runs the reference's own device functions on the host, for parity
// fixtures.  TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref/ from the
// reference's headers where they lie (include path REF_ROOT), never shipped.
//
// The loops reproduce the reference's kernels one thread per node:
//   RCSKernel              kernels.cu:119-131  (skip nodes where interior() is true)
//   JetBoundaryConditions  kernels.cu:102-114
//   InitJetBulk/InitJetInlet, InitStaticBubble, InitRTIDomain/InitRTIWalls  kernels.cu:22-96
#include "lbm.cuh"
#include "jet/jetIn.cuh"
#include "jet/boundary_conditions.cuh"
#include "bubble/bubbleIn.cuh"
#include "rti/rtiIn.cuh"

namespace {
MomentsDevice view(real_t *const *f) {
    MomentsDevice m;
    m.rhor = f[0]; m.rhob = f[1];
    m.ux = f[2]; m.uy = f[3]; m.uz = f[4];
    m.Pixx = f[5]; m.Pixy = f[6]; m.Piyy = f[7]; m.Piyz = f[8]; m.Pizz = f[9]; m.Pixz = f[10];
    return m;
}
void jet_bc(MomentsDevice b, const MomentsDevice a) {
    for (label_t z = 0; z < NZ; ++z)
        for (label_t x = 0; x < NX; ++x) {
            if (inlet_outlet_interior(x, z)) continue;
            inlet_bc_calculation(b, x, z);
            outlet_neumann_bc_calculation(b, a, x, z);
        }
}
} // namespace

extern "C" {
int ref_q() { return static_cast<int>(Q); }
int ref_real_bytes() { return static_cast<int>(sizeof(real_t)); }
int ref_dims(int *d) { d[0] = NX; d[1] = NY; d[2] = NZ; return 0; }

void ref_init_jet(real_t *const *A) {
    MomentsDevice a = view(A);
    for (label_t z = 0; z < NZ; ++z)
        for (label_t y = 0; y < NY; ++y)
            for (label_t x = 0; x < NX; ++x) init_jet_bulk(a, x, y, z);
    for (label_t z = 0; z < NZ; ++z)
        for (label_t x = 0; x < NX; ++x)
            if (!inlet_outlet_interior(x, z)) init_jet_inlet(a, x, z);
    jet_bc(a, a); // main.cu:26
}

void ref_init_bubble(real_t *const *A) {
    MomentsDevice a = view(A);
    for (label_t z = 0; z < NZ; ++z)
        for (label_t y = 0; y < NY; ++y)
            for (label_t x = 0; x < NX; ++x)
                if (!interior(x, y, z)) init_static_bubble(a, x, y, z);
}

void ref_init_rti(real_t *const *A) {
    MomentsDevice a = view(A);
    for (label_t z = 0; z < NZ; ++z)
        for (label_t y = 0; y < NY; ++y)
            for (label_t x = 0; x < NX; ++x) init_rti_domain(a, x, y, z);
    for (label_t z = 0; z < NZ; ++z)
        for (label_t x = 0; x < NX; ++x)
            if (!inlet_outlet_interior(x, z)) init_rti_y_walls(a, x, z);
}

// One step of main.cu:41-45 without the swap: RCS A -> B, then the boundary pass on B.
void ref_step(real_t *const *A, real_t *const *B, int do_rcs, int do_bc) {
    MomentsDevice a = view(A), b = view(B);
    if (do_rcs)
        for (label_t z = 0; z < NZ; ++z)
            for (label_t y = 0; y < NY; ++y)
                for (label_t x = 0; x < NX; ++x)
                    if (!interior(x, y, z)) RCS(a, b, x, y, z);
    if (do_bc) jet_bc(b, a);
}
}
