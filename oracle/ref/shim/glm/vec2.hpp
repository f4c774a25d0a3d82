// Forwarding header of the glm stand-in (test infrastructure only).
#pragma once
#include "glm_shim.hpp"
