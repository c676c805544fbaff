// Project-written stand-in (see glm/glm.hpp).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include "glm.hpp"
#include "gtc/matrix_transform.hpp"
