// fused-form stage kernel variants for transform length 2048
#include "stage_fused.cuh"

namespace pstd {

const StageVariant* stage_variants_fused_l(int L, int* n) {
    static const StageVariant v2048[] = {
        make_fused_variant<FCfg<2048, 4, 256, 2, 32, 64, 0, 0, 1>>("L2048 fused cs4 nt256 r32.2x32"),
        make_fused_variant<FCfg<2048, 2, 256, 3, 16, 16, 8>>("L2048 fused cs2 nt256 r16.16.8"),
        make_fused_variant<FCfg<2048, 2, 128, 4, 32, 64, 0, 0, 1>>("L2048 fused cs2 nt128 r32.2x32"),
        make_fused_variant<FCfg<2048, 4, 512, 1, 16, 16, 8>>("L2048 fused cs4 nt512 r16.16.8"),
    };
    switch (L) {
        case 2048: *n = 4; return v2048;
        default: *n = 0; return nullptr;
    }
}

}  // namespace pstd
