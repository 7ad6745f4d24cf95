// TMA-staged persistent stage kernel variants for transform lengths 128..512
#include "stage_tma.cuh"

namespace pstd {

const StageVariant* stage_variants_tma_a(int L, int* n) {
    static const StageVariant v128[] = {
        make_tma_variant<Cfg<128, 16, 256, 2, 16, 8>>("L128 tma cs16 nt256 r16.8"),
        make_tma_variant<Cfg<128, 8, 128, 4, 16, 8>>("L128 tma cs8 nt128 r16.8"),
    };
    static const StageVariant v256[] = {
        make_tma_variant<Cfg<256, 8, 256, 2, 16, 16>>("L256 tma cs8 nt256 r16.16"),
        make_tma_variant<Cfg<256, 4, 128, 4, 16, 16>>("L256 tma cs4 nt128 r16.16"),
    };
    static const StageVariant v512[] = {
        make_tma_variant<Cfg<512, 4, 256, 2, 8, 8, 8>>("L512 tma cs4 nt256 r8.8.8"),
        make_tma_variant<Cfg<512, 4, 128, 3, 32, 16>>("L512 tma cs4 nt128 r32.16"),
    };
    switch (L) {
        case 128: *n = 2; return v128;
        case 256: *n = 2; return v256;
        case 512: *n = 2; return v512;
        default: *n = 0; return nullptr;
    }
}

}  // namespace pstd
