/* timer.h -- wall-clock helpers (reference em2d/timer.h:21-50). */
#ifndef ZPIC_EM2D_TIMER_H
#define ZPIC_EM2D_TIMER_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
uint64_t timer_ticks(void);
double timer_interval_seconds(uint64_t start, uint64_t end);
double timer_cpu_seconds(void);
double timer_resolution(void);
#ifdef __cplusplus
}
#endif
#endif
