#ifndef SHIM_TIMER_H
#define SHIM_TIMER_H
#include <time.h>
struct Timer { struct timespec start_time, end_time; };
static inline void Start(struct Timer *t) { clock_gettime(CLOCK_MONOTONIC, &t->start_time); }
static inline void Stop(struct Timer *t) { clock_gettime(CLOCK_MONOTONIC, &t->end_time); }
static inline double Seconds(struct Timer *t)
{
    return (double)(t->end_time.tv_sec - t->start_time.tv_sec) +
           (double)(t->end_time.tv_nsec - t->start_time.tv_nsec) * 1e-9;
}
#endif
