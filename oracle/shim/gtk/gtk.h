/* Declaration-only stand-in for <gtk/gtk.h>.
 *
 * TEST INFRASTRUCTURE (oracle): MDZ's image_info.h names a handful of GLib /
 * GTK types in struct fields that the hot path never touches.  This header
 * gives them the same sizes (gboolean and guint32 are 32-bit integers,
 * GtkWidget is only used through a pointer) so that the unmodified hot-path
 * sources compile without GTK. */
#ifndef MDZ_SHIM_GTK_H
#define MDZ_SHIM_GTK_H

#include <stdint.h>
#include <stdlib.h>
#include <stdbool.h>

typedef int gboolean;
typedef uint32_t guint32;
typedef struct _GtkWidget GtkWidget;

#ifndef TRUE
#define TRUE 1
#endif
#ifndef FALSE
#define FALSE 0
#endif

#define g_free free

#endif
