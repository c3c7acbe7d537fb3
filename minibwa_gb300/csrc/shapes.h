// shapes.h -- thread-group shapes (G threads x K words each) instantiated for
// the extension DP kernel, ordered by window words G*K.  A pair whose
// reference n_col_ is c needs G*K >= 4*c (ksw2_extz2_sse.c:68); the score
// stores running past en0 land in the kernel's extra score-only slot.
// Without a tuned preference a pair runs on the first shape that holds its
// band, so among shapes of equal words the first is the default.  For 32-word
// bands (8,4) runs extd2 pairs of 100-300 nt at w=100 in 149.7 ns per pair on a
// GB300, (16,2), which fits five extd2 blocks per SM instead of four, in 170.4 ns.
#pragma once
#define KSW2G_SHAPES(X)                                                                              \
  X(0, 4, 3) X(1, 4, 4) X(2, 8, 3) X(3, 8, 4) X(4, 16, 2) X(5, 4, 8) X(6, 16, 3) X(7, 16, 4) X(8, 32, 4) \
  X(9, 32, 5) X(10, 32, 8)
#define KSW2G_NUM_SHAPES 11

// Block shapes (NW warps x K words a thread) of the block-split kernel (ext_split.cuh), ordered
// by window words 32*NW*K; the kernel is instantiated once per K and takes NW from the launch.
#define KSW2G_SPLIT_SHAPES(X)                                                                      \
  X(0, 2, 1) X(1, 3, 1) X(2, 4, 1) X(3, 5, 1) X(4, 6, 1) X(5, 8, 1) X(6, 10, 1) X(7, 12, 1) X(8, 16, 1) \
  X(9, 12, 2) X(10, 16, 2) X(11, 12, 4) X(12, 16, 4)
#define KSW2G_NUM_SPLIT_SHAPES 13
