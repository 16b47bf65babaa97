/* Oracle test infrastructure: empty stand-in (RabbitVar includes this
 * htslib header but uses none of its symbols). */
#ifndef RV_SHIM_KSTRING_H
#define RV_SHIM_KSTRING_H
#include <stddef.h>
#endif
