// Persistent single-launch time loop (odis_persistent.cu).
#pragma once

#include <cstddef>
#include <cuda_runtime.h>

#include "odis_device.cuh"

namespace odis {

constexpr int kPersistThreads = 512;

// Partition of the mesh over the CTAs of the persistent launch (device pointers).
// CTA b owns the faces forder[fstart[b] .. fstart[b+1]) and the cells
// corder[cstart[b] .. cstart[b+1]); the first fint[b] / cint[b] of them are
// interior (every face or cell they read is owned by b), the rest boundary.
struct PersistPlan {
    int P = 0;                    // CTAs (one per SM)
    int nf_max = 0, nc_max = 0;   // largest face / cell range of a CTA
    const int* fstart = nullptr;  // [P+1]
    const int* cstart = nullptr;  // [P+1]
    const int* fint = nullptr;    // [P] interior faces of each CTA
    const int* cint = nullptr;    // [P] interior cells of each CTA
    const int* forder = nullptr;  // [E] faces in CTA order (interior first)
    const int* corder = nullptr;  // [N] cells in CTA order
    const int* fpos = nullptr;    // [E] position of a face inside its CTA's range
    const int* cpos = nullptr;    // [N] position of a cell inside its CTA's range
    const int* fowner = nullptr;  // [E] owning CTA of each face
    const int* cowner = nullptr;  // [N] owning CTA of each cell
    const int* depA_ptr = nullptr;  // [P+1] CSR: CTAs whose cells / faces the face phase reads
    const int* depA = nullptr;
    const int* depC_ptr = nullptr;  // [P+1] CSR: CTAs whose faces the cell phase reads
    const int* depC = nullptr;
    unsigned* flag_e = nullptr;   // [P] face phases completed in the current run
    unsigned* flag_c = nullptr;   // [P] cell phases completed in the current run
    void* part = nullptr;         // [(n+1)][P] dissipation partials of a run (method type)
    unsigned spin_limit = 0;      // polls of one wait before it gives up (0: kSpinLimit, about a second)
    int withhold = -1;            // >= 0: this CTA publishes no step flags (failure-detection test hook)
};

size_t persist_smem_bytes(int value_bytes, int nf_max, int nc_max);
// 1 if one CTA with this plan's shared memory fits on an SM (and sets the attribute)
int persistent_fits(int precision, const PersistPlan& pl, int* max_blocks_per_sm);
// fc/cc/st point at FaceCoef<T>/CellCoef<T>/State<T> of the precision's type
int launch_persistent(int precision, const void* fc, const void* cc, const void* st, const StepConst& sc,
                      const PersistPlan& pl, int n, long long first, double* power, cudaStream_t s);

}  // namespace odis
