// Project-written stand-in (see glm/glm.hpp); nothing of it is used by the files compiled.
#pragma once
#include "../glm.hpp"
