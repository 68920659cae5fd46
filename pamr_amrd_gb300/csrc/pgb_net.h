/*
 * Internal layout of the learned initial guess (pgb_net.cu).
 *
 * Activations are BF16 in a channel-blocked, zero-padded layout: for
 * channel block cb (8 channels) the voxels of the level's volume padded by
 * one zero voxel on every side, x fastest, 8 channels per voxel (16 bytes):
 *     act[cb][margin + P][8],  P = (x+1) + Wp*((y+1) + Hp*(z+1)),
 *     Wp = W+2, Hp = H+2, Dp = D+2, x in [-1, W], ...
 * with a zero margin before and after the padded volume, so that the input
 * of every tap of every 128-voxel output tile is one contiguous run of
 * voxels per channel block, read with a 1-D bulk copy and consumed by
 * tcgen05.mma as a K-major operand without swizzle.
 */
#ifndef PGB_NET_H
#define PGB_NET_H

#include <stdint.h>

typedef struct {
   int W, H, D;          /* interior extents */
   int Wp, Hp, Dp;       /* padded extents */
   long plane;           /* Wp*Hp */
   long margin;          /* zero voxels before the padded volume (and after it) */
   long vtot;            /* voxels per channel block incl. both margins */
   long p0;              /* first padded index of the interior planes (z = 0) */
   int ntile;            /* 128-voxel output tiles covering planes z = 0..D-1 */
} pgb_lvgeom;

#endif
