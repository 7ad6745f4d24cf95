// fused-form stage kernel variants for transform lengths 512 and 1024
#include "stage_fused.cuh"

namespace pstd {

const StageVariant* stage_variants_fused_m(int L, int* n) {
    static const StageVariant v512[] = {
        make_fused_variant<FCfg<512, 8, 256, 3, 16, 32, 0, 0, 1>>("L512 fused cs8 nt256 r16.2x16"),
        make_fused_variant<FCfg<512, 8, 256, 2, 16, 32>>("L512 fused cs8 nt256 r16.32"),
        make_fused_variant<FCfg<512, 4, 128, 4, 16, 32>>("L512 fused cs4 nt128 r16.32"),
        make_fused_variant<FCfg<512, 8, 256, 3, 16, 8, 4>>("L512 fused cs8 nt256 r16.8.4"),
    };
    static const StageVariant v1024[] = {
        make_fused_variant<FCfg<1024, 4, 128, 4, 32, 32>>("L1024 fused cs4 nt128 r32.32"),
        make_fused_variant<FCfg<1024, 4, 256, 2, 16, 64, 0, 0, 1>>("L1024 fused cs4 nt256 r16.2x32"),
        make_fused_variant<FCfg<1024, 4, 256, 3, 16, 8, 8>>("L1024 fused cs4 nt256 r16.8.8"),
        make_fused_variant<FCfg<1024, 2, 128, 6, 16, 8, 8>>("L1024 fused cs2 nt128 r16.8.8"),
    };
    switch (L) {
        case 512: *n = 4; return v512;
        case 1024: *n = 4; return v1024;
        default: *n = 0; return nullptr;
    }
}

}  // namespace pstd
