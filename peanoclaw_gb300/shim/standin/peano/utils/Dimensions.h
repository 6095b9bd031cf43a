// Stand-in for peano/utils/Dimensions.h: the 2D build of PeanoClaw.
#ifndef PEANO_UTILS_DIMENSIONS_H_
#define PEANO_UTILS_DIMENSIONS_H_
#ifndef DIMENSIONS
#define DIMENSIONS 2
#endif
#define DIMENSIONS_TIMES_TWO (2 * DIMENSIONS)
#define TWO_POWER_D (1 << DIMENSIONS)
#endif
