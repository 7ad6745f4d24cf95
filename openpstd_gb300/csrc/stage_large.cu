// stage kernel variants for transform length 2048
#include "stage_kernel.cuh"

namespace pstd {

const StageVariant* stage_variants_large(int L, int* n) {
    static const StageVariant v2048[] = {
        make_variant<Cfg<2048, 4, 256, 3, 16, 16, 8>>("L2048 cs4 nt256 r16.16.8"),
        make_variant<Cfg<2048, 8, 512, 1, 16, 16, 8>>("L2048 cs8 nt512 r16.16.8"),
        make_variant<Cfg<2048, 4, 256, 3, 8, 8, 8, 4>>("L2048 cs4 nt256 r8.8.8.4"),
        make_variant<Cfg<2048, 4, 256, 1, 16, 16, 8, 0, 128>>("L2048 cs4 ws256+128 r16.16.8"),
        make_variant<Cfg<2048, 4, 256, 1, 16, 16, 8, 0, 384>>("L2048 cs4 ws256+384 r16.16.8"),
        make_pipe_variant<Cfg<2048, 2, 256, 1, 16, 16, 8>>("L2048 cs2 pipe256 r16.16.8"),
        make_pipe_variant<Cfg<2048, 1, 128, 2, 16, 16, 8>>("L2048 cs1 pipe128 r16.16.8"),
        make_variant<Cfg<2048, 4, 512, 2, 16, 16, 8>>("L2048 cs4 nt512 mb2 r16.16.8"),
        make_variant<Cfg<2048, 2, 256, 4, 16, 16, 8>>("L2048 cs2 nt256 mb4 r16.16.8"),
        make_sprev_variant<Cfg<2048, 4, 256, 2, 16, 16, 8>>("L2048 cs4 nt256 sprev r16.16.8"),
        make_sprev_variant<Cfg<2048, 2, 256, 4, 16, 16, 8>>("L2048 cs2 nt256 mb4 sprev r16.16.8"),
        make_variant<Cfg<2048, 4, 256, 3, 16, 16, 8, 0, 0, 0, 0, 1>>("L2048 cs4 nt256 r16.16.8 ctw"),
        make_variant<Cfg<2048, 4, 256, 2, 16, 16, 8, 0, 0, 0, 1, 1>>("L2048 cs4 nt256 mb2 r16.16.8 ilp ctw"),
        make_variant<Cfg<2048, 4, 256, 3, 8, 8, 8, 4, 0, 0, 0, 1>>("L2048 cs4 nt256 r8.8.8.4 ctw"),
        make_variant<Cfg<2048, 2, 256, 4, 16, 16, 8, 0, 0, 0, 0, 1>>("L2048 cs2 nt256 mb4 r16.16.8 ctw"),
        make_sprev_variant<Cfg<2048, 4, 256, 2, 16, 16, 8, 0, 0, 0, 0, 1>>("L2048 cs4 nt256 sprev r16.16.8 ctw"),
    };
    switch (L) {
        case 2048: *n = 16; return v2048;
        default: *n = 0; return nullptr;
    }
}

}  // namespace pstd
