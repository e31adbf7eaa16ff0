// Empty stand-in: the reference includes <glm/glm.hpp> from common.hpp but
// uses none of its symbols. Test infrastructure only.
#pragma once
