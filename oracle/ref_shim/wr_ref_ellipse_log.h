/* wr_ref_ellipse_log.h — declaration of the harness's record hook for the
 * anisotropic (elliptic) photon query of PhotonMap::throughputByDensityEstimation
 * (photonMap.cpp:384-652).  Test infrastructure only: oracle/Makefile inserts
 * three calls into its build copy of photonMap.cpp, one at each exit of that
 * branch, so that the reference's own ellipse (or its fallback to the round
 * kernel) can be compared with the C restatement on the same inputs.
 *
 * kind 0: the elliptic query (ratio and the ellipse frame's mX, mY given);
 * kind 1: fallback, eigenvectors within the |cs| or |sn| > 0.99 band;
 * kind 2: fallback, degenerate projection or Xi_s / Xi_f <= 1. */
#pragma once

#define WR_V3(v) (v).x, (v).y, (v).z

void wrEllipseLog(int kind, float ix, float iy, float iz, float nx, float ny, float nz, float sx, float sy, float sz,
                  float hx, float hy, float hz, float nu, float nv, float ratio, float ex, float ey, float ez,
                  float fx, float fy, float fz);
