/* Forwarding header with the reference's name (image_inpainting.h): the drop-in classes
 * are declared in nli_inpainting.hpp. */
#include "../nli_inpainting.hpp"
