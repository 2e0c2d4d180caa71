// ParlayLib header name used by the reference; the subset lives in parlay_shim.hpp.
#pragma once
#include "parlay_shim.hpp"
