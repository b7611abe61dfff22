/* empty stand-in: the reference base kernels include curand_kernel.h but use none of it */
#pragma once
