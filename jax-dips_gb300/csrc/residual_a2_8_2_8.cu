// DoubleMLP u- 2x8, u+ 2x8 (tanh): residual-path kernels for this shape.
#define DIPS_LM 2
#define DIPS_WM 8
#define DIPS_LP 2
#define DIPS_WP 8
#define DIPS_NS arch_2_8_2_8
#define DIPS_GETTER arch_ops_2_8_2_8
#include "residual_arch.cuh"
