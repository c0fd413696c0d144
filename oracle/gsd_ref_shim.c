/* Test infrastructure: a flat C interface over the reference's own GSD library
 * (hoomd/extern/gsd.c, compiled unmodified from the reference tree beside this shim by
 * oracle/build.py into oracle/_ref/libgsd_ref.so). The tests drive it through ctypes to read
 * files written by hoomd_gb300.gsd and to write files that hoomd_gb300.gsd must read. The handle
 * struct stays on the C side, so no struct layout crosses the boundary.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "gsd.h"

void* rg_open(const char* fname, int mode)
{
    /* mode 0: read only, 1: append */
    struct gsd_handle* h = (struct gsd_handle*)calloc(1, sizeof(struct gsd_handle));
    if (!h) return NULL;
    if (gsd_open(h, fname, mode == 0 ? GSD_OPEN_READONLY : GSD_OPEN_APPEND) != GSD_SUCCESS) {
        free(h);
        return NULL;
    }
    return h;
}

void* rg_create(const char* fname, const char* application, const char* schema,
                unsigned int major, unsigned int minor)
{
    struct gsd_handle* h = (struct gsd_handle*)calloc(1, sizeof(struct gsd_handle));
    if (!h) return NULL;
    if (gsd_create_and_open(h, fname, application, schema, gsd_make_version(major, minor),
                            GSD_OPEN_APPEND, 0) != GSD_SUCCESS) {
        free(h);
        return NULL;
    }
    return h;
}

int rg_close(void* h)
{
    int r = gsd_close((struct gsd_handle*)h);
    free(h);
    return r;
}

uint64_t rg_nframes(void* h) { return gsd_get_nframes((struct gsd_handle*)h); }

/* header fields: versions, application and schema (64 bytes each) */
void rg_header(void* h, uint32_t* gsd_version, uint32_t* schema_version, char* application,
               char* schema)
{
    struct gsd_handle* g = (struct gsd_handle*)h;
    *gsd_version = g->header.gsd_version;
    *schema_version = g->header.schema_version;
    memcpy(application, g->header.application, 64);
    memcpy(schema, g->header.schema, 64);
}

/* 1 and the chunk's N, M, type when the chunk exists in the frame, else 0 */
int rg_find(void* h, uint64_t frame, const char* name, uint64_t* N, uint32_t* M, uint8_t* type)
{
    const struct gsd_index_entry* e = gsd_find_chunk((struct gsd_handle*)h, frame, name);
    if (!e) return 0;
    *N = e->N;
    *M = e->M;
    *type = e->type;
    return 1;
}

int rg_read(void* h, uint64_t frame, const char* name, void* data)
{
    const struct gsd_index_entry* e = gsd_find_chunk((struct gsd_handle*)h, frame, name);
    if (!e) return -1000;
    return gsd_read_chunk((struct gsd_handle*)h, data, e);
}

int rg_write(void* h, const char* name, int type, uint64_t N, uint32_t M, const void* data)
{
    return gsd_write_chunk((struct gsd_handle*)h, name, (enum gsd_type)type, N, M, 0, data);
}

int rg_end_frame(void* h) { return gsd_end_frame((struct gsd_handle*)h); }

/* the next name after prev (NULL for the first) that starts with match, or NULL */
const char* rg_match(void* h, const char* match, const char* prev)
{
    return gsd_find_matching_chunk_name((struct gsd_handle*)h, match, prev);
}
