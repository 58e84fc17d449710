// Stand-in for the OpenCV core header, for compiling the reference's own
// sources into the oracle's reference build (test infrastructure only).  The
// reference functions that build uses do not touch OpenCV; their headers
// only name its types in declarations of other functions, so the types are
// declared here and never defined or used.
#ifndef TDM_REF_OPENCV_CORE_SHIM_HPP
#define TDM_REF_OPENCV_CORE_SHIM_HPP
namespace cv {
class Mat;
class Size;
class String;
}  // namespace cv
#define CV_64F 6
#define CV_8U 0
#define CV_8UC1 0
#define CV_32F 5
#endif
