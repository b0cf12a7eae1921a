// ref_vti.cpp -- writes one VTI image with the reference's own writer (io/vtiWriter.cuh,
// write_vti) from raw FP32 fields.  TEST INFRASTRUCTURE ONLY: it produces the golden file the
// VTI-format test compares the library's writer with (tests/golden/make_golden.py).
//   ref_vti <in.raw> <out.vti>   in.raw: rhor, rhob, ux, uy, uz, NX*NY*NZ floats each
#include <cstdio>
#include <vector>

#include "io/vtiWriter.cuh"

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    std::vector<real_t> buf(5 * static_cast<size_t>(Ncells));
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    const size_t got = std::fread(buf.data(), sizeof(real_t), buf.size(), f);
    std::fclose(f);
    if (got != buf.size()) return 4;
    LbmHost h;
    h.rhor = buf.data();
    h.rhob = buf.data() + Ncells;
    h.ux = buf.data() + 2 * static_cast<size_t>(Ncells);
    h.uy = buf.data() + 3 * static_cast<size_t>(Ncells);
    h.uz = buf.data() + 4 * static_cast<size_t>(Ncells);
    write_vti(argv[2], h);
    return 0;
}
