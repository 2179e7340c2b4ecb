/* random.h -- the em1d drop-in's generator: the same multiply-with-carry
 * pair and polar Box-Muller deviates as em1d/random.h:21-28 (identical to
 * the em2d API). */
#include "../em2d/random.h"
