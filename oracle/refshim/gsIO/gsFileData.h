// Test-only empty stand-in: the solver headers compiled for the CPU oracle include it but use
// nothing from it.
#pragma once
#include <gsCore/gsLinearAlgebra.h>
