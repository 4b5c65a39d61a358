/* Dump hook linked into the reference `c` backend programs built under
 * oracle/_ref/ (test infrastructure only; never part of the product).
 *
 * A generated program (src/backend/CPrinter.cpp:189-233) is patched with one
 * call to abl_ref_dump() at the top of every timestep, and compiled with
 * `-Dsave=abl_ref_save` so that its final save() also dumps.  Each dump writes,
 * for every agent type in agents_info (CPrinter.cpp:295-302), the agent count
 * as uint64 followed by every agent packed member by member in declaration
 * order without padding (bool 1 byte, int 4, float 8, float2 16, float3 24 in
 * FP64 mode; 4/8/12 under LIBABL_USE_FLOAT).  The output file is named by the
 * ABL_DUMP environment variable. */
#include "libabl.h"
#include <stdio.h>
#include <stdint.h>
#include <stdlib.h>

static size_t member_size(type_id t) {
	switch (t) {
		case TYPE_BOOL: return sizeof(bool);
		case TYPE_INT: return sizeof(int);
		case TYPE_FLOAT: return sizeof(abl_float);
		case TYPE_FLOAT2: return sizeof(float2);
		case TYPE_FLOAT3: return sizeof(float3);
		default: return 0;
	}
}

static size_t record_size(const type_info *info) {
	while (info->type != TYPE_END) ++info;
	return info->offset;
}

static FILE *dump_file(void) {
	static FILE *f = NULL;
	if (!f) {
		const char *path = getenv("ABL_DUMP");
		if (!path) return NULL;
		f = fopen(path, "wb");
	}
	return f;
}

void abl_ref_dump(void *agents, const agent_info *info) {
	FILE *f = dump_file();
	if (!f) return;
	for (; info->name; info++) {
		dyn_array *arr = (dyn_array *) ((char *) agents + info->offset);
		uint64_t n = arr->len;
		size_t rec = record_size(info->info);
		fwrite(&n, sizeof n, 1, f);
		for (size_t i = 0; i < arr->len; i++) {
			const char *agent = (const char *) arr->values + rec * i;
			for (const type_info *m = info->info; m->type != TYPE_END; m++) {
				fwrite(agent + m->offset, member_size(m->type), 1, f);
			}
		}
	}
	fflush(f);
}

void abl_ref_save(void *agents, const agent_info *info, const char *path, save_type type) {
	(void) path;
	(void) type;
	abl_ref_dump(agents, info);
}
