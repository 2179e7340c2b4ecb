/* timer.h -- wall-clock helpers of the em1d drop-in (em1d/timer.h:21-50,
 * identical to the em2d API). */
#include "../em2d/timer.h"
