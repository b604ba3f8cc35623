// direct.h stand-in (src/s3d_pt.cpp:13 includes it; nothing from it is used on the oracle path).
#pragma once
