// Stand-in for the CUDA runtime header in the host emulation of the sieve.
#pragma once
#include "sieve_shim.h"
