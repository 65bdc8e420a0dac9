/* stand-in for the obsolete <sys/timeb.h> (removed from glibc); the
   reference's timing helpers (routines.cu:186-199) only need ftime(). */
#pragma once
#include <time.h>
struct timeb { time_t time; unsigned short millitm; short timezone, dstflag; };
static inline int ftime(struct timeb *tb) {
  struct timespec ts; clock_gettime(CLOCK_REALTIME, &ts);
  tb->time = ts.tv_sec; tb->millitm = (unsigned short)(ts.tv_nsec / 1000000);
  tb->timezone = 0; tb->dstflag = 0; return 0;
}
