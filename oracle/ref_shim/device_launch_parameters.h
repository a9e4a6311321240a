// Host shim (see cuda_runtime.h in this folder).
#pragma once
#include "cuda_runtime.h"
