/* A stand-in for the few libxml2 tree declarations pi-qmc's XMLParser and the
 * GPU tag parser use (the image has no libxml2).  TEST INFRASTRUCTURE: an
 * element is a name, attribute pairs, children and a next sibling, enough
 * for tests/adapters/parser_check.cc to build an input fragment by hand. */
#ifndef PIMC_STUB_LIBXML_TREE_H
#define PIMC_STUB_LIBXML_TREE_H
#include <stdlib.h>
#include <string.h>

typedef unsigned char xmlChar;
#define BAD_CAST (xmlChar*)

typedef enum { XML_ELEMENT_NODE = 1, XML_TEXT_NODE = 3 } xmlElementType;

typedef struct _xmlNode {
  xmlElementType type;
  const xmlChar* name;
  struct _xmlNode* children;
  struct _xmlNode* next;
  const char* const* attrs; /* name, value, name, value, ..., 0 */
} xmlNode;
typedef xmlNode* xmlNodePtr;

/* The attribute's value as a new string (free with xmlFree), or 0. */
static inline xmlChar* xmlGetProp(const xmlNode* node, const xmlChar* name) {
  for (const char* const* a = node->attrs; a && a[0]; a += 2)
    if (strcmp(a[0], (const char*)name) == 0) {
      char* v = (char*)malloc(strlen(a[1]) + 1);
      strcpy(v, a[1]);
      return (xmlChar*)v;
    }
  return 0;
}
static inline void xmlFree(void* p) { free(p); }
#endif
