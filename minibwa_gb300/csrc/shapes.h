// shapes.h -- thread-group shapes (G threads x K words each) instantiated for
// the extension DP kernel.  A pair whose reference n_col_ is c needs
// G*K >= 4*(c+1) window words (ksw2_extz2_sse.c:68 plus one block that holds
// the score stores running past en0).
#pragma once
#define KSW2G_SHAPES(X) X(0, 4, 4) X(1, 8, 3) X(2, 8, 5) X(3, 16, 4) X(4, 32, 4) X(5, 32, 8)
#define KSW2G_NUM_SHAPES 6
