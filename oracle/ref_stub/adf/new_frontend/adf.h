/* Forwards to the project's minimal <adf.h> stand-in (see ../../adf.h). */
#pragma once
#include "../../adf.h"
