// stage kernel variants for transform lengths 32 .. 256
#include "stage_kernel.cuh"

namespace pstd {

const StageVariant* stage_variants_small(int L, int* n) {
    static const StageVariant v32[] = {
        make_variant<Cfg<32, 16, 64, 8, 8, 4>>("L32 cs16 nt64 r8.4"),
    };
    static const StageVariant v64[] = {
        make_variant<Cfg<64, 16, 128, 6, 8, 8>>("L64 cs16 nt128 r8.8"),
    };
    static const StageVariant v128[] = {
        make_variant<Cfg<128, 16, 128, 6, 16, 8>>("L128 cs16 nt128 r16.8"),
        make_variant<Cfg<128, 8, 64, 8, 16, 8>>("L128 cs8 nt64 r16.8"),
        make_variant<Cfg<128, 16, 128, 1, 16, 8, 0, 0, 64>>("L128 cs16 ws128+64 r16.8"),
        make_pipe_variant<Cfg<128, 16, 128, 2, 16, 8>>("L128 cs16 pipe128 r16.8"),
        make_pipe_variant<Cfg<128, 8, 64, 4, 16, 8>>("L128 cs8 pipe64 r16.8"),
        make_variant<Cfg<128, 16, 128, 8, 16, 8>>("L128 cs16 nt128 mb8 r16.8"),
        make_sprev_variant<Cfg<128, 16, 128, 6, 16, 8>>("L128 cs16 nt128 sprev r16.8"),
        make_variant<Cfg<128, 16, 128, 6, 16, 8, 0, 0, 0, 0, 0, 1>>("L128 cs16 nt128 r16.8 ctw"),
        make_variant<Cfg<128, 16, 128, 8, 16, 8, 0, 0, 0, 0, 0, 1>>("L128 cs16 nt128 mb8 r16.8 ctw"),
        make_sprev_variant<Cfg<128, 16, 128, 6, 16, 8, 0, 0, 0, 0, 0, 1>>("L128 cs16 nt128 sprev r16.8 ctw"),
        make_pipe_variant<Cfg<128, 8, 64, 4, 16, 8, 0, 0, 0, 0, 0, 1>>("L128 cs8 pipe64 r16.8 ctw"),
    };
    static const StageVariant v256[] = {
        make_variant<Cfg<256, 16, 256, 3, 16, 16>>("L256 cs16 nt256 r16.16"),
        make_variant<Cfg<256, 8, 128, 5, 16, 16>>("L256 cs8 nt128 r16.16"),
        make_variant<Cfg<256, 16, 256, 1, 16, 16, 0, 0, 128>>("L256 cs16 ws256+128 r16.16"),
        make_pipe_variant<Cfg<256, 8, 128, 2, 16, 16>>("L256 cs8 pipe128 r16.16"),
        make_variant<Cfg<256, 16, 256, 4, 16, 16>>("L256 cs16 nt256 mb4 r16.16"),
        make_sprev_variant<Cfg<256, 16, 256, 3, 16, 16>>("L256 cs16 nt256 sprev r16.16"),
        make_variant<Cfg<256, 16, 256, 4, 16, 16, 0, 0, 0, 0, 0, 1>>("L256 cs16 nt256 mb4 r16.16 ctw"),
        make_variant<Cfg<256, 8, 128, 5, 16, 16, 0, 0, 0, 0, 0, 1>>("L256 cs8 nt128 r16.16 ctw"),
        make_sprev_variant<Cfg<256, 16, 256, 3, 16, 16, 0, 0, 0, 0, 0, 1>>("L256 cs16 nt256 sprev r16.16 ctw"),
    };
    switch (L) {
        case 32: *n = 1; return v32;
        case 64: *n = 1; return v64;
        case 128: *n = 11; return v128;
        case 256: *n = 9; return v256;
        default: *n = 0; return nullptr;
    }
}

}  // namespace pstd
