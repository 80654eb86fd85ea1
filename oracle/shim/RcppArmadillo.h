// RcppArmadillo.h -- forwards to the project-written API shim (test infrastructure only).
#include "sdg_shim.hpp"
