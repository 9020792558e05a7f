/* stub: GL type names only, so that the compute sources compile headless */
#include "glew.h"
