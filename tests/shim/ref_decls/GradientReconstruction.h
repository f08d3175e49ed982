// Stand-in for the reference's include/GradientReconstruction.h: the scheme
// selector only (include/GradientReconstruction.h:12-15).
#ifndef GRADIENTRECONSTRUCTION_H_INCLUDED
#define GRADIENTRECONSTRUCTION_H_INCLUDED
enum class GradientScheme { GreenGauss, LeastSquares };
#endif
