// Translation unit of qbatch_impl.cuh: adjoint_f32.
#define BGB_QB_ADJ_F32
#include "qbatch_impl.cuh"
