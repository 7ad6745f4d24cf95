// fused-form stage kernel variants for transform lengths 4096 and 8192
#include "stage_fused.cuh"

namespace pstd {

const StageVariant* stage_variants_fused_h(int L, int* n) {
    static const StageVariant v4096[] = {
        make_fused_variant<FCfg<4096, 2, 256, 2, 32, 2, 64, 0, 1>>("L4096 fused cs2 nt256 r32.2.2x32"),
        make_fused_variant<FCfg<4096, 2, 512, 1, 16, 16, 16>>("L4096 fused cs2 nt512 r16.16.16"),
        make_fused_variant<FCfg<4096, 1, 256, 3, 16, 16, 16>>("L4096 fused cs1 nt256 r16.16.16"),
    };
    static const StageVariant v8192[] = {
        make_fused_variant<FCfg<8192, 1, 256, 2, 32, 8, 32>>("L8192 fused cs1 nt256 r32.8.32"),
        make_fused_variant<FCfg<8192, 1, 512, 1, 16, 16, 32>>("L8192 fused cs1 nt512 r16.16.32"),
        make_fused_variant<FCfg<8192, 1, 256, 2, 32, 4, 64, 0, 1>>("L8192 fused cs1 nt256 r32.4.2x32"),
    };
    switch (L) {
        case 4096: *n = 3; return v4096;
        case 8192: *n = 3; return v8192;
        default: *n = 0; return nullptr;
    }
}

}  // namespace pstd
