/* Timer for the reference build (project-written stand-in, test infrastructure). */
#ifndef ORC_TIMER_H
#define ORC_TIMER_H
#include <sys/time.h>
inline double get_full_time() { struct timeval tv; gettimeofday(&tv, 0); return (double)tv.tv_sec * 100.0 + (double)tv.tv_usec / 10000.0; }
class Timer { double t0_; public: Timer() : t0_(get_full_time()) {} double elapsed() const { return (get_full_time() - t0_) / 100.0; } void restart() { t0_ = get_full_time(); } };
#endif
