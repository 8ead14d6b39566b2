// Oracle-build stand-in: all parameter types live in ParamSlot.h.
#pragma once
#include "mmcore/param/ParamSlot.h"
