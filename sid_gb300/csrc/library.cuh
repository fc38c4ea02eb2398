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

// Forward projections of the staged boxes into the library rows: FP32
// lenslet taps (library.cu) or the tensor-core windows (libtc.cu).  Both
// leave `st` unsynchronised.
int lib_run_direct(sid_plan* p, const char* who, const std::vector<LibBox>& boxes, float* out, int out_layout,
                   cudaStream_t st);
int lib_run_spectral(sid_plan* p, const char* who, const std::vector<LibBox>& boxes, float* out, int out_layout,
                     cudaStream_t st);

// LibBox lattice window fields (s0..t1) of a box whose x0..z1 are set
void lib_box_window(const sid_plan* p, LibBox& b);

}  // namespace sid
