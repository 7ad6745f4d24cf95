// stage kernel variants for transform lengths 4096 and 8192
#include "stage_tc5.cuh"

namespace pstd {

const StageVariant* stage_variants_huge(int L, int* n) {
    static const StageVariant v4096[] = {
        make_variant<Cfg<4096, 2, 256, 3, 16, 16, 16>>("L4096 cs2 nt256 r16.16.16"),
        make_variant<Cfg<4096, 4, 512, 1, 16, 16, 16>>("L4096 cs4 nt512 r16.16.16"),
        make_variant<Cfg<4096, 1, 256, 1, 16, 16, 16, 0, 128>>("L4096 cs1 ws256+128 r16.16.16"),
        make_pipe_variant<Cfg<4096, 1, 256, 1, 16, 16, 16>>("L4096 cs1 pipe256 r16.16.16"),
        make_variant<Cfg<4096, 2, 512, 2, 16, 16, 16>>("L4096 cs2 nt512 mb2 r16.16.16"),
        make_variant<Cfg<4096, 2, 256, 3, 16, 16, 16, 0, 0, 0, 0, 1>>("L4096 cs2 nt256 r16.16.16 ctw"),
        make_variant<Cfg<4096, 2, 256, 2, 16, 16, 16, 0, 0, 0, 1, 1>>("L4096 cs2 nt256 mb2 r16.16.16 ilp ctw"),
        make_variant<Cfg<4096, 1, 256, 2, 16, 16, 16, 0, 0, 1>>("L4096 cs1 nt256 r16.16.16 bf16x3"),
    };
    static const StageVariant v8192[] = {
        make_variant<Cfg<8192, 1, 256, 3, 16, 16, 8, 4>>("L8192 cs1 nt256 r16.16.8.4"),
        make_variant<Cfg<8192, 2, 512, 1, 16, 16, 8, 4>>("L8192 cs2 nt512 r16.16.8.4"),
        make_variant<Cfg<8192, 1, 512, 2, 16, 16, 8, 4>>("L8192 cs1 nt512 mb2 r16.16.8.4"),
        make_variant<Cfg<8192, 1, 256, 2, 32, 16, 16>>("L8192 cs1 nt256 mb2 r32.16.16"),
        make_variant<Cfg<8192, 1, 256, 3, 16, 16, 8, 4, 0, 0, 0, 1>>("L8192 cs1 nt256 r16.16.8.4 ctw"),
        make_variant<Cfg<8192, 2, 512, 1, 16, 16, 8, 4, 0, 0, 0, 1>>("L8192 cs2 nt512 r16.16.8.4 ctw"),
        make_variant<Cfg<8192, 1, 256, 2, 16, 16, 8, 4, 0, 0, 1, 1>>("L8192 cs1 nt256 mb2 r16.16.8.4 ilp ctw"),
        make_variant<Cfg<8192, 1, 256, 2, 16, 16, 16, 2, 0, 1>>("L8192 cs1 nt256 r16.16.16.2 bf16x3"),
        make_tc5_variant<Cfg<8192, 1, 256, 1, 16, 16, 16, 2>>("L8192 cs1 nt256 r16.16.16.2 tcgen05 tf32x3"),
    };
    switch (L) {
        case 4096: *n = 8; return v4096;
        case 8192: *n = 9; return v8192;
        default: *n = 0; return nullptr;
    }
}

}  // namespace pstd
