// RAFT header name mapped onto the stand-ins in refshim_raft.hpp.
#pragma once
#include "../../refshim_raft.hpp"
