/* random.h -- Marsaglia multiply-with-carry generator and polar Box-Muller
 * deviates, as the reference's em2d/random.h:21-28.  The first seed argument
 * sets the "w" state (the reference's random.c:25-29).  The state is per
 * host thread: a single-threaded program sees the reference's process-global
 * generator. */
#ifndef ZPIC_EM2D_RANDOM_H
#define ZPIC_EM2D_RANDOM_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
void set_rand_seed(uint32_t m_w_, uint32_t m_z_);
uint32_t rand_uint32(void);
double rand_norm(void);
/* addition: seeds and drops the cached deviate, the state of a newly
 * started process (no counterpart in the reference) */
void rand_seed_fresh(uint32_t m_w_, uint32_t m_z_);
#ifdef __cplusplus
}
#endif
#endif
