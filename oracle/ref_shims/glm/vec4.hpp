// Forwarding header of the project-written glm stand-in (test infrastructure).
#pragma once
#include "detail_vec.hpp"
