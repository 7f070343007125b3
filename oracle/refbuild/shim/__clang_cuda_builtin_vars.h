// Clang-only CUDA header named by one reference source; nvcc needs nothing from it.
#pragma once
