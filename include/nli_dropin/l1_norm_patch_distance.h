/* Forwarding header with the reference's name (l1_norm_patch_distance.h): the drop-in classes
 * are declared in nli_inpainting.hpp. */
#include "../nli_inpainting.hpp"
