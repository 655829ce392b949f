// ImageUtilities header name used by the reference sources; everything is in pdt_iu_shim.h.
#pragma once
#include "pdt_iu_shim.h"
