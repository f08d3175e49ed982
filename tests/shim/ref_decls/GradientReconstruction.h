// Stand-in for the reference's include/GradientReconstruction.h: the scheme
// selector (include/GradientReconstruction.h:12-15) and the per-cell
// gradient struct (include/GradientReconstruction.h:19-22).
#ifndef GRADIENTRECONSTRUCTION_H_INCLUDED
#define GRADIENTRECONSTRUCTION_H_INCLUDED
enum class GradientScheme { GreenGauss, LeastSquares };
struct Gradient2 {
    double dphidx = 0.0;
    double dphidy = 0.0;
};
#endif
