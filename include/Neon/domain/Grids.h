// All grids of the GB300 Neon API (one partition, one GPU).
#pragma once
#include "Neon/domain/bGrid.h"
#include "Neon/domain/dGrid.h"
#include "Neon/domain/eGrid.h"
