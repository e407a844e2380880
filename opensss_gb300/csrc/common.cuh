// Shared definitions for the sm_103a TOF-SSS engine (libsss300.so).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sss300.h"

namespace sss {

// Device-side error bits, OR-ed into the caller's status word; the host maps
// them to the SSS_ERR_* codes of sss300.h after the stream is synchronised.
enum DeviceError : int32_t {
    kErrOverrun = 1 << 0,    // traversal would pass Nx+Ny+Nz voxels (reference: IndexError)
    kErrTofRange = 1 << 1,   // TOF table index above 8000 (reference: IndexError)
    kErrEnergy = 1 << 2,     // scattered-energy row outside the 2000-row tables
    kErrVoxel = 1 << 3,      // linear voxel index outside the volume (Nx != Ny case)
    kErrCapacity = 1 << 4,   // an internal list capacity was exceeded
    kErrEvent = 1 << 5,      // a list-mode event outside the sinogram tables (reference: IndexError)
    kErrNonFinite = 1 << 6,  // a detector pair's slice term came out infinite or NaN
    kErrTable = 1 << 7,      // a caller's index table (sampled rings or crystals, LOR, cell or
                             // slice table) holds an entry outside its range; nothing is read there
    // not an error: set by the tail mask's pre-pass when the map has a negative
    // or NaN value (its line integrals can then shrink); sss_status_code ignores it
    kNoteMapSigned = 1 << 30,
};

constexpr int kTofEntries = 8001;  // -4000..4000 ps, SingleScatterSimulationTOF.py:145-147
constexpr int kTimeRange = 4000;

__device__ __forceinline__ void raise_error(int32_t* status, int32_t bits)
{
    if (status) atomicOr(status, bits);
}

// 2^x with the SFU (ex2.approx.ftz.f32, max rel. error about 2^-22).
__device__ __forceinline__ float ex2(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

}  // namespace sss

// Host helpers shared by the entry points (defined in api.cu and sss.cu).
int sss_set_error(int code, const char* fmt, ...);
int sss_check_launch(const char* what);
int sss_internal_validate(const sss_tof_problem* p);
// Enumerates p's scatter points into points (capacity entries of 4 doubles);
// counts[0] = total, counts[1 + i] = points of sampled slice i (zeroed by the caller).
int sss_internal_scatter_points(const sss_tof_problem* p, double* points, long long capacity,
                                unsigned long long* counts, cudaStream_t st);
