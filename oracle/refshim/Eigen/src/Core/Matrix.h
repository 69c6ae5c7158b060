// Stand-in for Eigen/src/Core/Matrix.h (viscositymodel.cpp:2); see Eigen/Core.
#include "../../Core"
