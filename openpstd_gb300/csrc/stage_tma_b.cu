// TMA-staged persistent stage kernel variants for transform lengths 1024 and 2048
#include "stage_tma.cuh"

namespace pstd {

const StageVariant* stage_variants_tma_b(int L, int* n) {
    static const StageVariant v1024[] = {
        make_tma_variant<Cfg<1024, 4, 256, 2, 16, 8, 8>>("L1024 tma cs4 nt256 r16.8.8"),
        make_tma_variant<Cfg<1024, 2, 128, 4, 16, 8, 8>>("L1024 tma cs2 nt128 r16.8.8"),
        make_tma_variant<Cfg<1024, 4, 512, 1, 16, 8, 8>>("L1024 tma cs4 nt512 r16.8.8"),
    };
    static const StageVariant v2048[] = {
        make_tma_variant<Cfg<2048, 2, 256, 2, 16, 16, 8>>("L2048 tma cs2 nt256 r16.16.8"),
        make_tma_variant<Cfg<2048, 2, 256, 2, 8, 8, 8, 4>>("L2048 tma cs2 nt256 r8.8.8.4"),
        make_tma_variant<Cfg<2048, 4, 512, 1, 16, 16, 8>>("L2048 tma cs4 nt512 r16.16.8"),
    };
    switch (L) {
        case 1024: *n = 3; return v1024;
        case 2048: *n = 3; return v2048;
        default: *n = 0; return nullptr;
    }
}

}  // namespace pstd
