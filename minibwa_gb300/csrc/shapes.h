// shapes.h -- thread-group shapes (G threads x K words each) instantiated for
// the extension DP kernel, ordered by window words G*K.  A pair whose
// reference n_col_ is c needs G*K >= 4*c (ksw2_extz2_sse.c:68); the score
// stores running past en0 land in the kernel's extra score-only slot.
#pragma once
#define KSW2G_SHAPES(X)                                                                              \
  X(0, 4, 3) X(1, 4, 4) X(2, 8, 3) X(3, 8, 4) X(4, 4, 8) X(5, 16, 3) X(6, 16, 4) X(7, 32, 4) X(8, 32, 5) \
  X(9, 32, 8)
#define KSW2G_NUM_SHAPES 10
