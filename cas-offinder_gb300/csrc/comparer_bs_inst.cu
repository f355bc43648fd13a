// One (ROW, NK, CONC) instance set of the bit-sliced comparer kernels; the
// build compiles this file once per set with COF_BS_ROW, COF_BS_NK and
// COF_BS_CONC defined.
#include "comparer_bs.cuh"

#if !defined(COF_BS_ROW) || !defined(COF_BS_NK) || !defined(COF_BS_CONC)
#error "COF_BS_ROW, COF_BS_NK and COF_BS_CONC must be defined"
#endif

template bool cof::bs::dispatch_s<COF_BS_ROW, COF_BS_NK, (COF_BS_CONC != 0)>(
    int, const cof::GenomeView&, const uint32_t*, const uint32_t*, uint64_t, const uint32_t*, const uint32_t*, uint32_t,
    uint32_t, bool, uint32_t, uint32_t*, uint64_t*, unsigned long long*, uint64_t, int, cudaStream_t);
