// TEST INFRASTRUCTURE: printing is not used by the solver sources.
#pragma once
#include "xtensor.hpp"
