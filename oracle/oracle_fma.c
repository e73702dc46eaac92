/*
 * TEST INFRASTRUCTURE ONLY -- part of the CPU oracle, never linked into the
 * product library.  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg may load it.
 *
 * The reference rotates point sets with BLAS matrix products:
 *   tools/utilities.py:315   rotated = np.dot(coords, R.T)      (atoms)
 *   tools/detector.py:71,113,155  R @ np.vstack([x, y, z])      (detector)
 * OpenBLAS evaluates each output element of these 3-term dot products as the
 * left-to-right fused chain  fma(p2, R[i][2], fma(p1, R[i][1], p0 * R[i][0])).
 * That order is pinned by tests/golden (generated from the reference itself);
 * this file states it explicitly with C99 fma() so the oracle gives the same
 * bits on any host, independent of which BLAS kernel numpy happens to load.
 *
 * Build with -ffp-contract=off so the compiler adds no fusions of its own.
 */
#include <math.h>
#include <stdint.h>

/* out[k*3+i] = fma(p[2], R[i*3+2], fma(p[1], R[i*3+1], p[0]*R[i*3+0])),
 * p = pts + 3k, R row-major 3x3. */
void oracle_rotate_rows(const double *pts, int64_t n, const double *R,
                        double *out) {
  for (int64_t k = 0; k < n; ++k) {
    const double *p = pts + 3 * k;
    double o0 = fma(p[2], R[2], fma(p[1], R[1], p[0] * R[0]));
    double o1 = fma(p[2], R[5], fma(p[1], R[4], p[0] * R[3]));
    double o2 = fma(p[2], R[8], fma(p[1], R[7], p[0] * R[6]));
    out[3 * k + 0] = o0;
    out[3 * k + 1] = o1;
    out[3 * k + 2] = o2;
  }
}

/* Same chain on split component arrays (x, y, z), as R @ vstack([x,y,z]). */
void oracle_rotate_xyz(const double *x, const double *y, const double *z,
                       int64_t n, const double *R, double *ox, double *oy,
                       double *oz) {
  for (int64_t k = 0; k < n; ++k) {
    double a = x[k], b = y[k], c = z[k];
    double o0 = fma(c, R[2], fma(b, R[1], a * R[0]));
    double o1 = fma(c, R[5], fma(b, R[4], a * R[3]));
    double o2 = fma(c, R[8], fma(b, R[7], a * R[6]));
    ox[k] = o0;
    oy[k] = o1;
    oz[k] = o2;
  }
}
