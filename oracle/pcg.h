// PCG32 sampler, restating the reference's PCGSampler (src/core/sampler.h:13-91)
// and interleave_32bit (src/util/hash.h:12-27).  Test infrastructure only.
#pragma once
#include <cstdint>
#include <cstring>

namespace oracle {

inline uint32_t interleave_32bit(uint32_t x, uint32_t y) {
    x &= 0x0000ffffu;
    y &= 0x0000ffffu;
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    y = (y | (y << 8)) & 0x00FF00FFu;
    y = (y | (y << 4)) & 0x0F0F0F0Fu;
    y = (y | (y << 2)) & 0x33333333u;
    y = (y | (y << 1)) & 0x55555555u;
    return x | (y << 1);
}

struct Pcg {
    static constexpr uint64_t kMult = 0x5851f42d4c957f2dULL;
    uint64_t state = 0x853c49e6748fea9bULL;
    uint64_t inc = 0xda3e39cb94b95bdbULL;

    // sampler.h:22-28
    void set_seed(uint64_t initstate, uint64_t initseq = 1) {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next_u32();
        state += initstate;
        next_u32();
    }
    // sampler.h:30-34
    void set_pixel_sample(uint32_t px, uint32_t py, uint32_t sample_index) {
        set_seed(interleave_32bit(px, py), sample_index);
    }
    // sampler.h:42-55
    void advance(int64_t delta) {
        uint64_t cur_mult = kMult, cur_plus = inc, acc_mult = 1u, acc_plus = 0u;
        while (delta > 0) {
            if (delta & 1) {
                acc_mult *= cur_mult;
                acc_plus = acc_plus * cur_mult + cur_plus;
            }
            cur_plus = (cur_mult + 1) * cur_plus;
            cur_mult *= cur_mult;
            delta /= 2;
        }
        state = acc_mult * state + acc_plus;
    }
    // sampler.h:58-64
    uint32_t next_u32() {
        uint64_t old = state;
        state = old * kMult + inc;
        uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((~rot + 1u) & 31));
    }
    // sampler.h:77-86
    float get1d() {
        uint32_t u = (next_u32() >> 9) | 0x3f800000u;
        float f;
        std::memcpy(&f, &u, 4);
        return f - 1.0f;
    }
};

}  // namespace oracle
