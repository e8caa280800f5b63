/* Forwarding header with the reference's name (patch_non_local_medians.h): the drop-in classes
 * are declared in nli_inpainting.hpp. */
#include "../nli_inpainting.hpp"
