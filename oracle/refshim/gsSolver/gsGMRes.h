// Test-only stand-in: see gsLinearOperator.h.
#pragma once
#include <gsSolver/gsLinearOperator.h>
