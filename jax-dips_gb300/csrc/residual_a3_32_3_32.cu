// DoubleMLP u- 3x32, u+ 3x32 (tanh): residual-path kernels for this shape.
#define DIPS_LM 3
#define DIPS_WM 32
#define DIPS_LP 3
#define DIPS_WP 32
#define DIPS_NS arch_3_32_3_32
#define DIPS_GETTER arch_ops_3_32_3_32
#include "residual_arch.cuh"
