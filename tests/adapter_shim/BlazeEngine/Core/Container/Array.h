// Test infrastructure: see BlazeEngine/AdapterShimCommon.h.
#pragma once
#include "BlazeEngine/AdapterShimCommon.h"
