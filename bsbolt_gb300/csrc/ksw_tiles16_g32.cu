// ksw_tiles16_g32.cu -- extension kernels with 32 lanes (a warp) per job, 16-bit cells two to a
// register (ksw_group16.cuh), for the shapes with an even C (see ksw_tiles.cuh).
#include "ksw_tiles_impl.cuh"

KswTileLaunch ksw_tiles16_g32(int C)
{
    switch (C) {
    case 6: return ksw_tile16_launch<3, 32>;
    case 8: return ksw_tile16_launch<4, 32>;
    case 10: return ksw_tile16_launch<5, 32>;
    case 12: return ksw_tile16_launch<6, 32>;
    case 14: return ksw_tile16_launch<7, 32>;
    case 16: return ksw_tile16_launch<8, 32>;
    case 20: return ksw_tile16_launch<10, 32>;
    case 24: return ksw_tile16_launch<12, 32>;
    case 28: return ksw_tile16_launch<14, 32>;
    case 32: return ksw_tile16_launch<16, 32>;
    default: return nullptr;
    }
}
