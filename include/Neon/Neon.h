// Umbrella header of the GB300 Neon API (Neon::init, core types, Backend,
// containers). Grids: "Neon/domain/dGrid.h", "Neon/domain/bGrid.h";
// "Neon/skeleton/Skeleton.h"; solver: "Neon/solver/linear/krylov/CG.h";
// LBM containers on the sm_103a kernels: "Neon/gb300/lbm.h".
#pragma once
#include "Neon/core/core.h"
#include "Neon/set/Backend.h"
#include "Neon/set/Containter.h"
