// acq_bounds.cuh — device index checks of the debug build (-DACQ_BOUNDS_CHECK).
//
// In the checked build every instrumented global-memory access must fall inside a buffer the
// library registered: its own device allocations and the caller's device input of the current
// request. An access outside all of them is skipped and recorded (first failing site, its
// address, number of failures) in a device table instead of faulting; acq_fetch_results then
// returns ACQ_ERR_CUDA with the site and address. In the normal build ACQ_BC(ptr, site) expands
// to nothing and the statement after it runs unconditionally.
//
// Each translation unit that launches kernels holds its own copy of the table pointer (a
// __constant__ symbol), set by the host through acq_bounds_set_table_<unit>.
#pragma once

#include <cstdint>

namespace acq {

constexpr int kBcMaxRanges = 1024;

struct BoundsTable {
    unsigned long long base[kBcMaxRanges];
    unsigned long long end[kBcMaxRanges];   // one past the last byte
    int n;                                  // registered ranges
    int err_site;                           // first failing site, 0 = none
    unsigned long long err_addr;            // its address
    unsigned long long hits;                // accesses skipped
};

#ifdef ACQ_BOUNDS_CHECK
static __constant__ BoundsTable* c_bounds_table;

__device__ __noinline__ inline bool bc_ok(const void* p, unsigned bytes, int site) {
    BoundsTable* t = c_bounds_table;
    if (!t) return true;
    const unsigned long long a = reinterpret_cast<unsigned long long>(p), e = a + bytes;
    const int n = *static_cast<volatile int*>(&t->n);
    for (int i = 0; i < n; ++i)
        if (a >= t->base[i] && e <= t->end[i]) return true;
    if (atomicCAS(&t->err_site, 0, site) == 0) t->err_addr = a;
    atomicAdd(&t->hits, 1ull);
    return false;
}
// checks the range [p, p + bytes) once (bulk copies, vector loads)
#define ACQ_BC_RANGE(p, bytes, site) if (::acq::bc_ok((p), static_cast<unsigned>(bytes), (site)))
#define ACQ_BC(ptr, site) if (::acq::bc_ok((ptr), static_cast<unsigned>(sizeof(*(ptr))), (site)))
#define ACQ_BC_SET_TABLE_IMPL(name)                                                          \
    cudaError_t name(void* table) {                                                          \
        ::acq::BoundsTable* t = static_cast<::acq::BoundsTable*>(table);                     \
        return cudaMemcpyToSymbol(::acq::c_bounds_table, &t, sizeof(t));                    \
    }
#else
#define ACQ_BC_RANGE(p, bytes, site)
#define ACQ_BC(ptr, site)
#define ACQ_BC_SET_TABLE_IMPL(name) \
    cudaError_t name(void*) { return cudaSuccess; }
#endif

}  // namespace acq
