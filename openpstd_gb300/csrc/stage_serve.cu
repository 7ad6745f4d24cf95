// stage_serve.cu -- the stage kernel configurations of the serving loop's
// per-length persistent form: one per transform length, each compiled with
// the device-count persistent loop (stage_kernel_dev).  They are the
// configurations the autotuner picks on batches of scenes like the serving
// stream (cells log-uniform 64x64 .. 1024x768, 50-cell PML), so a server
// gets tuned arithmetic without timing variants on live scenes.
#include "stage_kernel.cuh"

namespace pstd {

const StageVariant* serve_variant(int L) {
    static const StageVariant v[] = {
        make_dev_variant<Cfg<32, 16, 64, 8, 8, 4>>("L32 cs16 nt64 r8.4 (serving)"),
        make_dev_variant<Cfg<64, 16, 128, 6, 8, 8>>("L64 cs16 nt128 r8.8 (serving)"),
        make_dev_variant<Cfg<128, 16, 128, 8, 16, 8, 0, 0, 0, 0, 0, 1>>("L128 cs16 nt128 mb8 r16.8 ctw (serving)"),
        make_dev_variant<Cfg<256, 16, 256, 4, 16, 16>>("L256 cs16 nt256 mb4 r16.16 (serving)"),
        make_dev_variant<Cfg<512, 8, 256, 4, 8, 8, 8, 0, 0, 0, 0, 1>>("L512 cs8 nt256 mb4 r8.8.8 ctw (serving)"),
        make_dev_variant<Cfg<1024, 4, 256, 4, 16, 8, 8, 0, 0, 0, 0, 1>>("L1024 cs4 nt256 mb4 r16.8.8 ctw (serving)"),
        make_dev_variant<Cfg<2048, 2, 256, 4, 16, 16, 8, 0, 0, 0, 0, 1>>("L2048 cs2 nt256 mb4 r16.16.8 ctw (serving)"),
        make_dev_variant<Cfg<4096, 2, 256, 3, 16, 16, 16, 0, 0, 0, 0, 1>>("L4096 cs2 nt256 r16.16.16 ctw (serving)"),
        make_dev_variant<Cfg<8192, 1, 256, 3, 16, 16, 8, 4, 0, 0, 0, 1>>("L8192 cs1 nt256 r16.16.8.4 ctw (serving)"),
    };
    for (const StageVariant& x : v)
        if (x.L == L) return &x;
    return nullptr;
}

}  // namespace pstd
