// stage kernel variants for transform lengths 512 and 1024
#include "stage_kernel.cuh"

namespace pstd {

const StageVariant* stage_variants_mid(int L, int* n) {
    static const StageVariant v512[] = {
        make_variant<Cfg<512, 8, 256, 3, 8, 8, 8>>("L512 cs8 nt256 r8.8.8"),
        make_variant<Cfg<512, 4, 128, 6, 8, 8, 8>>("L512 cs4 nt128 r8.8.8"),
        make_variant<Cfg<512, 8, 256, 1, 8, 8, 8, 0, 128>>("L512 cs8 ws256+128 r8.8.8"),
        make_pipe_variant<Cfg<512, 4, 128, 2, 8, 8, 8>>("L512 cs4 pipe128 r8.8.8"),
        make_variant<Cfg<512, 8, 256, 4, 8, 8, 8>>("L512 cs8 nt256 mb4 r8.8.8"),
        make_variant<Cfg<512, 8, 128, 4, 32, 16>>("L512 cs8 nt128 mb4 r32.16"),
        make_sprev_variant<Cfg<512, 8, 256, 3, 8, 8, 8>>("L512 cs8 nt256 sprev r8.8.8"),
        make_variant<Cfg<512, 8, 256, 4, 8, 8, 8, 0, 0, 0, 0, 1>>("L512 cs8 nt256 mb4 r8.8.8 ctw"),
        make_variant<Cfg<512, 8, 256, 3, 16, 8, 4, 0, 0, 0, 0, 1>>("L512 cs8 nt256 r16.8.4 ctw"),
        make_sprev_variant<Cfg<512, 8, 256, 3, 8, 8, 8, 0, 0, 0, 0, 1>>("L512 cs8 nt256 sprev r8.8.8 ctw"),
    };
    static const StageVariant v1024[] = {
        make_variant<Cfg<1024, 8, 256, 3, 16, 8, 8>>("L1024 cs8 nt256 r16.8.8"),
        make_variant<Cfg<1024, 4, 256, 3, 16, 8, 8>>("L1024 cs4 nt256 r16.8.8"),
        make_variant<Cfg<1024, 4, 128, 5, 16, 8, 8>>("L1024 cs4 nt128 r16.8.8"),
        make_variant<Cfg<1024, 8, 256, 1, 16, 8, 8, 0, 128>>("L1024 cs8 ws256+128 r16.8.8"),
        make_variant<Cfg<1024, 8, 256, 1, 16, 8, 8, 0, 384>>("L1024 cs8 ws256+384 r16.8.8"),
        make_pipe_variant<Cfg<1024, 4, 256, 1, 16, 8, 8>>("L1024 cs4 pipe256 r16.8.8"),
        make_pipe_variant<Cfg<1024, 2, 128, 2, 16, 8, 8>>("L1024 cs2 pipe128 r16.8.8"),
        make_variant<Cfg<1024, 4, 256, 4, 16, 8, 8>>("L1024 cs4 nt256 mb4 r16.8.8"),
        make_variant<Cfg<1024, 2, 128, 8, 16, 8, 8>>("L1024 cs2 nt128 mb8 r16.8.8"),
        make_variant<Cfg<1024, 4, 128, 4, 32, 32>>("L1024 cs4 nt128 mb4 r32.32"),
        make_variant<Cfg<1024, 8, 256, 2, 32, 32>>("L1024 cs8 nt256 mb2 r32.32"),
        make_sprev_variant<Cfg<1024, 4, 256, 3, 16, 8, 8>>("L1024 cs4 nt256 sprev r16.8.8"),
        make_sprev_variant<Cfg<1024, 4, 256, 4, 16, 8, 8>>("L1024 cs4 nt256 mb4 sprev r16.8.8"),
        make_sprev_variant<Cfg<1024, 8, 256, 2, 32, 32>>("L1024 cs8 nt256 mb2 sprev r32.32"),
        make_variant<Cfg<1024, 4, 256, 3, 16, 8, 8, 0, 0, 0, 0, 1>>("L1024 cs4 nt256 r16.8.8 ctw"),
        make_variant<Cfg<1024, 8, 256, 3, 16, 8, 8, 0, 0, 0, 0, 1>>("L1024 cs8 nt256 r16.8.8 ctw"),
        make_variant<Cfg<1024, 8, 256, 2, 16, 8, 8, 0, 0, 0, 1, 1>>("L1024 cs8 nt256 mb2 r16.8.8 ilp ctw"),
        make_variant<Cfg<1024, 4, 256, 4, 16, 8, 8, 0, 0, 0, 0, 1>>("L1024 cs4 nt256 mb4 r16.8.8 ctw"),
        make_sprev_variant<Cfg<1024, 4, 256, 3, 16, 8, 8, 0, 0, 0, 0, 1>>("L1024 cs4 nt256 sprev r16.8.8 ctw"),
    };
    switch (L) {
        case 512: *n = 10; return v512;
        case 1024: *n = 19; return v1024;
        default: *n = 0; return nullptr;
    }
}

}  // namespace pstd
