// Bounds-checked build.  Compiled with -DSPHX_CHECK, the kernels test the indices they
// read through (neighbour-list entries against the number of records they index, cell-list
// ranges against the cell offsets, cell indices against the mesh) before the access; a
// failed test is counted and its first occurrence recorded (site and offending value), and
// the access is skipped, so a bad index never reaches memory.  sphx_check_violations reads
// and clears the record.  Without -DSPHX_CHECK every test is the constant `true` and the
// kernels compile to the unchecked code.  The reference has no such build: its loops index
// std::vector / SYCL buffers unchecked.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace sphx
{
// Sites of the index tests (the high 16 bits of the recorded first violation); the macro
// SPHX_CHECKED(ok, site, value) takes the bare enumerator name.
enum CheckSite : unsigned
{
    kCheckListEntry = 1,  // neighbour-list entry beyond the records it indexes (the staged
                          // records of a tile window for the tiled sweeps)
    kCheckCellRange = 2,  // cell-list range with begin > end or end beyond the particles
    kCheckCellIndex = 3   // cell index outside the mesh
};

// Violations recorded by one translation unit: reads (and with reset clears) its counters.
using CheckReader = int (*)(unsigned long long *count, unsigned long long *first, bool reset);
// Registers a translation unit's reader (checked builds); returns the number registered.
int check_register(CheckReader reader);
} // namespace sphx

#ifdef SPHX_CHECK
namespace
{
// One record per translation unit (whole-program device code: each unit owns its symbols).
__device__ unsigned long long g_check_count;
__device__ unsigned long long g_check_first;

__device__ __forceinline__ bool check_record(bool ok, unsigned site, unsigned long long value)
{
    if (!ok && atomicAdd(&g_check_count, 1ull) == 0ull)
        g_check_first = (static_cast<unsigned long long>(site) << 48) | (value & 0xffffffffffffull);
    return ok;
}

int check_read(unsigned long long *count, unsigned long long *first, bool reset)
{
    if (cudaMemcpyFromSymbol(count, g_check_count, sizeof(*count)) != cudaSuccess ||
        cudaMemcpyFromSymbol(first, g_check_first, sizeof(*first)) != cudaSuccess)
        return 1;
    if (reset)
    {
        const unsigned long long zero = 0;
        if (cudaMemcpyToSymbol(g_check_count, &zero, sizeof(zero)) != cudaSuccess ||
            cudaMemcpyToSymbol(g_check_first, &zero, sizeof(zero)) != cudaSuccess)
            return 1;
    }
    return 0;
}

const int g_check_registered = ::sphx::check_register(check_read);
} // namespace
#define SPHX_CHECKED(ok, site, value) ::check_record((ok), ::sphx::site, static_cast<unsigned long long>(value))
#else
#define SPHX_CHECKED(ok, site, value) true
#endif
