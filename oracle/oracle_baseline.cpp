// CPU baseline (placeholder, filled in with the Newton/PCG restatement).
#include "bartels_oracle.hpp"
