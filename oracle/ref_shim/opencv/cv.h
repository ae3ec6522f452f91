/* Minimal stand-in for the OpenCV 1.x C API: only what the reference's
 * mcRenderer.cpp and film.cpp name.  The harness never displays or loads
 * images; these buffers back the PFM helper only. */
#pragma once
#include <cstdlib>
#include <cstring>
#define IPL_DEPTH_32F 32
#define IPL_DEPTH_8U 8
struct CvSize { int width, height; };
static inline CvSize cvSize(int w, int h) { CvSize s; s.width = w; s.height = h; return s; }
struct CvScalar { double val[4]; };
struct IplImage { int width, height, nChannels, depth; char* imageData; };
static inline IplImage* cvCreateImage(CvSize s, int depth, int ch) {
    IplImage* im = new IplImage;
    im->width = s.width; im->height = s.height; im->nChannels = ch; im->depth = depth;
    size_t bytes = (size_t)s.width * s.height * ch * (depth == IPL_DEPTH_32F ? 4 : 1);
    im->imageData = (char*)calloc(bytes ? bytes : 1, 1);
    return im;
}
static inline void cvReleaseImage(IplImage** im) { if (im && *im) { free((*im)->imageData); delete *im; *im = 0; } }
static inline CvSize cvGetSize(const IplImage* im) { return cvSize(im->width, im->height); }
static inline CvScalar cvGet2D(const IplImage*, int, int) { CvScalar s = {{0, 0, 0, 0}}; return s; }
static inline void cvSet2D(IplImage*, int, int, CvScalar) {}
static inline IplImage* cvLoadImage(const char*, int) { return cvCreateImage(cvSize(1, 1), IPL_DEPTH_8U, 3); }
