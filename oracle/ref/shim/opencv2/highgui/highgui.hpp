// Stand-in for the OpenCV highgui header (see ../core/core.hpp).
#ifndef TDM_REF_OPENCV_HIGHGUI_SHIM_HPP
#define TDM_REF_OPENCV_HIGHGUI_SHIM_HPP
#include "../core/core.hpp"
#endif
