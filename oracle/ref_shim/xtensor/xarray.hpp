// TEST INFRASTRUCTURE: see xtensor.hpp.
#pragma once
#include "xtensor.hpp"
