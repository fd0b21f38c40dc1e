// Translation unit of qbatch_impl.cuh: stats.
#define BGB_QB_STATS
#include "qbatch_impl.cuh"
