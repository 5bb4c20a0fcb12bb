// DoubleMLP u- 1x1, u+ 2x10 (tanh): residual-path kernels for this shape.
#define DIPS_LM 1
#define DIPS_WM 1
#define DIPS_LP 2
#define DIPS_WP 10
#define DIPS_NS arch_1_1_2_10
#define DIPS_GETTER arch_ops_1_1_2_10
#include "residual_arch.cuh"
