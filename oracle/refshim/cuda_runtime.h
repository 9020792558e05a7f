/* shim: see shim.h */
#include "shim.h"
