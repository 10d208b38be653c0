/* Forwarding stand-in: every apegrunt name the SuperDCA solve headers use is
 * declared in the test oracle's apegrunt/Alignment.h stand-in. */
#pragma once
#include "apegrunt/Alignment.h"
