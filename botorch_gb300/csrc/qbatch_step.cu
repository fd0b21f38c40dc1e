// Translation unit of qbatch_impl.cuh: step.
#define BGB_QB_STEP
#include "qbatch_impl.cuh"
