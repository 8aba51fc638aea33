/* Declaration-only stand-in for <gtk/gtk.h>.
 *
 * TEST INFRASTRUCTURE (oracle): MDZ's image_info.h and the palette code name
 * a handful of GLib / GTK types in struct fields and locals that the hot
 * path and the colouring functions never hand to GTK.  This header gives
 * them the same sizes (gboolean, gint, guint, guint32 are 32-bit integers,
 * guint8 an unsigned byte, gdouble a double, widgets only pointers) so that
 * the unmodified sources compile without GTK. */
#ifndef MDZ_SHIM_GTK_H
#define MDZ_SHIM_GTK_H

#include <stdint.h>
#include <stdlib.h>
#include <stdbool.h>

typedef int gboolean;
typedef uint32_t guint32;
typedef uint8_t guint8;
typedef unsigned int guint;
typedef int gint;
typedef double gdouble;
typedef void* gpointer;
typedef struct _GtkWidget GtkWidget;
typedef struct _GtkWindow GtkWindow;

/* GLib's byte-order macros (palette.h packs RGB by them) */
#define G_LITTLE_ENDIAN 1234
#define G_BIG_ENDIAN 4321
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_BIG_ENDIAN__
#define G_BYTE_ORDER G_BIG_ENDIAN
#else
#define G_BYTE_ORDER G_LITTLE_ENDIAN
#endif

#ifndef TRUE
#define TRUE 1
#endif
#ifndef FALSE
#define FALSE 0
#endif

#define g_free free

#endif
