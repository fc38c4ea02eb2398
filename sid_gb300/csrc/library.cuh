// library.cuh -- neuron boxes shared by the two library generators
// (library.cu: FP32 lenslet taps; libtc.cu: tensor-core spectral windows).
#pragma once

#include <cstdint>
#include <vector>

#include "sid_internal.cuh"

namespace sid {

struct LibBox {
    int x0, x1, y0, y1, z0, z1;  // 0-based half-open box
    int off;                     // offset of the packed sub-volume
    int ncomp;                   // components averaged
    int s0, s1, t0, t1;          // output lenslet window (half-open, clipped to the lattice)
};

// The neurons' boxes (generate_LFM_library_GPU.m:68-88) on the host, uploaded
// to p->ws[3]; their averaged sub-volumes packed back to back into p->ws[2]
// (packed[off + dx + bw (dy + bh dz)] = mean over the neuron's components);
// p->ws[1] holds the staged pointers and ids.  `who` names the caller in errors.
int lib_stage(sid_plan* p, const char* who, const float* const* recon, int64_t n_comp, const double* centers,
              const uint8_t* neur_id, int64_t n_neur, int64_t neur_rad, double axial, std::vector<LibBox>& boxes,
              cudaStream_t st);

}  // namespace sid
