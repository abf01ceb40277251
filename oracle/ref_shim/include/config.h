/* TEST INFRASTRUCTURE ONLY: the four autoconf results the reference sources
 * read (src/unordered_map_dfn.h:1-9, src/wndchrm_src/TrainingSet.h). */
#define HAVE_UNORDERED_MAP 1
#define HAVE_UNORDERED_SET 1
#define PACKAGE_VERSION "1.60"
#define PACKAGE_STRING "wndchrm 1.60"
