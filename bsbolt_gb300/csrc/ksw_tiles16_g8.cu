// ksw_tiles16_g8.cu -- extension kernels with 8 lanes per job, 16-bit cells two to a
// register (ksw_group16.cuh), for the shapes with an even C (see ksw_tiles.cuh).
#include "ksw_tiles_impl.cuh"

KswTileLaunch ksw_tiles16_g8(int C)
{
    switch (C) {
    case 6: return ksw_tile16_launch<3, 8>;
    case 8: return ksw_tile16_launch<4, 8>;
    case 10: return ksw_tile16_launch<5, 8>;
    case 12: return ksw_tile16_launch<6, 8>;
    case 14: return ksw_tile16_launch<7, 8>;
    case 16: return ksw_tile16_launch<8, 8>;
    case 18: return ksw_tile16_launch<9, 8>;
    default: return nullptr;
    }
}
