// Translation unit of qbatch_impl.cuh: adjoint_f64.
#define BGB_QB_ADJ_F64
#include "qbatch_impl.cuh"
