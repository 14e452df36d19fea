// ksw_tiles16_g16.cu -- extension kernels with 16 lanes per job, 16-bit cells two to a
// register (ksw_group16.cuh), for the shapes with an even C (see ksw_tiles.cuh).
#include "ksw_tiles_impl.cuh"

KswTileLaunch ksw_tiles16_g16(int C)
{
    switch (C) {
    case 6: return ksw_tile16_launch<3, 16>;
    case 8: return ksw_tile16_launch<4, 16>;
    case 10: return ksw_tile16_launch<5, 16>;
    case 12: return ksw_tile16_launch<6, 16>;
    case 14: return ksw_tile16_launch<7, 16>;
    case 16: return ksw_tile16_launch<8, 16>;
    default: return nullptr;
    }
}
