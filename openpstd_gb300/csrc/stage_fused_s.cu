// fused-form stage kernel variants for transform lengths 128 and 256
#include "stage_fused.cuh"

namespace pstd {

const StageVariant* stage_variants_fused_s(int L, int* n) {
    static const StageVariant v128[] = {
        make_fused_variant<FCfg<128, 16, 256, 3, 8, 16>>("L128 fused cs16 nt256 r8.16"),
        make_fused_variant<FCfg<128, 8, 128, 5, 8, 16>>("L128 fused cs8 nt128 r8.16"),
        make_fused_variant<FCfg<128, 16, 256, 2, 4, 32>>("L128 fused cs16 nt256 r4.32"),
        make_fused_variant<FCfg<128, 16, 256, 3, 4, 32, 0, 0, 1>>("L128 fused cs16 nt256 r4.2x16"),
    };
    static const StageVariant v256[] = {
        make_fused_variant<FCfg<256, 8, 128, 5, 16, 16>>("L256 fused cs8 nt128 r16.16"),
        make_fused_variant<FCfg<256, 16, 256, 3, 16, 16>>("L256 fused cs16 nt256 r16.16"),
        make_fused_variant<FCfg<256, 8, 256, 2, 8, 32>>("L256 fused cs8 nt256 r8.32"),
    };
    switch (L) {
        case 128: *n = 4; return v128;
        case 256: *n = 3; return v256;
        default: *n = 0; return nullptr;
    }
}

}  // namespace pstd
