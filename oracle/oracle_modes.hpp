// Oracle: reference-mode shapes, elevation modes and coloring (filled in below).
#pragma once
#include "oracle_core.hpp"
