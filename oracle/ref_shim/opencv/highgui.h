/* Minimal stand-in for OpenCV highgui: the reference's window calls are not
 * used by the oracle harness (no display on this machine). */
#pragma once
#include "cv.h"
static inline void cvNamedWindow(const char*) {}
static inline void cvShowImage(const char*, const IplImage*) {}
static inline int cvWaitKey(int) { return -1; }
static inline int cvSaveImage(const char*, const IplImage*) { return 0; }
static inline void cvDestroyWindow(const char*) {}
