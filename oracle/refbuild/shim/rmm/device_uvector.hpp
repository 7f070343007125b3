// RMM header name mapped onto the stand-ins in refshim_rmm.hpp.
#pragma once
#include "../refshim_rmm.hpp"
