// dvec.h stand-in (include/s3d_typedef.h:281 includes it; none of its classes are used).
#pragma once
