// The per-step basis angle of the reference (LinAlgebra::base_projection,
// src/linear_algebra.cpp:3-11): a std::mt19937 seeded with one glibc rand() value, one
// uniform_real_distribution<double>(0,1) draw r, angle = M_2_PI * r. The stream is seeded
// once by srand(seed) (src/main.cpp:211). Using the same C library and libstdc++ calls
// keeps the sequence identical to the reference on any glibc host.
#include <cmath>
#include <cstdlib>
#include <random>

#include "fg_host.h"

extern "C" {

void fg_rng_seed(unsigned int seed) { srand(seed); }

double fg_rng_angle(void) {
    std::mt19937 gen(rand());
    std::uniform_real_distribution<> distrib(0.0, 1.0);
    const double r = distrib(gen);
    return M_2_PI * r;
}

}  // extern "C"
