/* Forwarding header with the reference's name (a_patch_distance.h): the drop-in classes
 * are declared in nli_inpainting.hpp. */
#include "../nli_inpainting.hpp"
