/* ipow for the reference build (project-written stand-in, test infrastructure).
 * Repeated multiplication from 1.0; linal's own ipow is unpinned. */
#ifndef ORC_POW_H
#define ORC_POW_H
inline double ipow(double x, int n) { double r = 1.0; for (int i = 0; i < n; ++i) r *= x; return r; }
#endif
