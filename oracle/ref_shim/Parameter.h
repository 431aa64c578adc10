/* The reference includes "Parameter.h" while the file is parameter.h (cpp/parameter.h); on a
 * case-sensitive file system this forwards to it. */
#include "parameter.h"
