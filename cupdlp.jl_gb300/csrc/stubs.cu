// stubs.cu — entry points not implemented yet: they fail loudly with NOT_SUPPORTED.
#include "problem.h"

extern "C" {
}
