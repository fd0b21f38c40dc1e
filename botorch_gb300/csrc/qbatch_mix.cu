// Translation unit of qbatch_impl.cuh: mix.
#define BGB_QB_MIX
#include "qbatch_impl.cuh"
