// C entry points for the PCG known-answer tests (test infrastructure only).
#include "oracle.h"
#include "pcg.h"

extern "C" void oracle_pcg_floats(uint32_t px, uint32_t py, uint32_t sample_index,
                                  int64_t advance_by, int count, float *out) {
    oracle::Pcg p;
    p.set_pixel_sample(px, py, sample_index);
    p.advance(advance_by);
    for (int i = 0; i < count; ++i) out[i] = p.get1d();
}

extern "C" void oracle_pcg_u32(uint64_t initstate, uint64_t initseq, int count, uint32_t *out) {
    oracle::Pcg p;
    p.set_seed(initstate, initseq);
    for (int i = 0; i < count; ++i) out[i] = p.next_u32();
}

extern "C" uint32_t oracle_interleave_32bit(uint32_t x, uint32_t y) {
    return oracle::interleave_32bit(x, y);
}
