/* Stand-in for libxml2's xpath.h (see tree.h beside it).  TEST INFRASTRUCTURE. */
#ifndef PIMC_STUB_LIBXML_XPATH_H
#define PIMC_STUB_LIBXML_XPATH_H
#include "tree.h"
typedef struct _xmlXPathContext {
  xmlNodePtr node;
} xmlXPathContext;
typedef xmlXPathContext* xmlXPathContextPtr;
#endif
