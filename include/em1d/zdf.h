/* zdf.h -- the ZDF diagnostic file interface of the em1d drop-in; the
 * reference's em1d/zdf.h is the same interface as em2d's. */
#include "../em2d/zdf.h"
