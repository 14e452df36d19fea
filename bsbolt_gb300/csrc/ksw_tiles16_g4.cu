// ksw_tiles16_g4.cu -- extension kernels with 4 lanes per job, 16-bit cells two to a
// register (ksw_group16.cuh), for the shapes with an even C (see ksw_tiles.cuh).
#include "ksw_tiles_impl.cuh"

KswTileLaunch ksw_tiles16_g4(int C)
{
    switch (C) {
    case 2: return ksw_tile16_launch<1, 4>;
    case 4: return ksw_tile16_launch<2, 4>;
    case 6: return ksw_tile16_launch<3, 4>;
    case 8: return ksw_tile16_launch<4, 4>;
    case 10: return ksw_tile16_launch<5, 4>;
    case 12: return ksw_tile16_launch<6, 4>;
    case 14: return ksw_tile16_launch<7, 4>;
    case 16: return ksw_tile16_launch<8, 4>;
    case 20: return ksw_tile16_launch<10, 4>;
    case 24: return ksw_tile16_launch<12, 4>;
    case 28: return ksw_tile16_launch<14, 4>;
    case 32: return ksw_tile16_launch<16, 4>;
    default: return nullptr;
    }
}
