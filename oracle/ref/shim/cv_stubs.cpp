// Definitions for the OpenCV C-API calls the reference makes for its preview
// window and image buffers (MCRenderer.cpp, Renderer.cpp). The oracle renders
// headless: images are plain heap buffers, window calls do nothing.
#include <opencv/cv.h>
#include <opencv/highgui.h>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "IntersectionGPU.h"

std::vector<SimpleShape*> IntersectionGPU::shapes;
std::vector<IntersectionGPU::Ray> IntersectionGPU::rayList;

extern "C" {
IplImage* cvCreateImage(CvSize size, int depth, int channels) {
  IplImage* im = (IplImage*)calloc(1, sizeof(IplImage));
  int bytes = (depth & 255) / 8;
  im->nSize = sizeof(IplImage);
  im->width = size.width;
  im->height = size.height;
  im->nChannels = channels;
  im->depth = depth;
  im->widthStep = size.width * channels * bytes;
  im->imageSize = im->widthStep * size.height;
  im->imageData = (char*)calloc(1, im->imageSize);
  im->imageDataOrigin = im->imageData;
  return im;
}
void cvReleaseImage(IplImage** im) {
  if (im && *im) { free((*im)->imageData); free(*im); *im = nullptr; }
}
void cvShowImage(const char*, const CvArr*) {}
int cvWaitKey(int) { return -1; }
void cvSetMouseCallback(const char*, CvMouseCallback, void*) {}
void cvLine(CvArr*, CvPoint, CvPoint, CvScalar, int, int, int) {}
void cvCircle(CvArr*, CvPoint, int, CvScalar, int, int, int) {}
void cvRectangle(CvArr*, CvPoint, CvPoint, CvScalar, int, int, int) {}
void cvConvertScale(const CvArr*, CvArr*, double, double) {}
void cvDestroyAllWindows(void) {}
int cvNamedWindow(const char*, int) { return 0; }
}
