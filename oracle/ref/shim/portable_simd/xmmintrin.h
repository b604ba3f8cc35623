// Forwards to the portable stand-in (oracle only).
#pragma once
#include "immintrin.h"
