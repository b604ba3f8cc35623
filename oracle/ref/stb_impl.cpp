// Instantiates the reference's vendored stb_image_write (external/stb, public
// domain) for PathTracer::Capture.  Oracle only.
#define STB_IMAGE_WRITE_IMPLEMENTATION
#include <stb_image_write.h>
