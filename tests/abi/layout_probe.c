/* Prints the size and field offsets of the chunk-set types, compiled once
 * against the reference's src/chunkset.h and once against
 * include/voxgpu_chunkset.h (tests/test_abi.py compares the two). */
#include <stddef.h>
#include <stdio.h>
#ifdef USE_REFERENCE
#include "chunkset.h"
#else
#include "voxgpu_chunkset.h"
#endif
#define F(T, f) printf("%s.%s %zu\n", #T, #f, offsetof(struct T, f))
int main(void)
{
	printf("ChunkSet %zu\nChunkMD %zu\nGeometrySVL %zu\nGeometryMesh %zu\n", sizeof(struct ChunkSet),
	       sizeof(struct ChunkMD), sizeof(struct GeometrySVL), sizeof(struct GeometryMesh));
	F(ChunkSet, count); F(ChunkSet, root); F(ChunkSet, root_bitw); F(ChunkSet, max); F(ChunkSet, max_bitw);
	F(ChunkSet, gsvl); F(ChunkSet, gmesh); F(ChunkSet, chunks); F(ChunkSet, null_chunk);
	F(ChunkSet, shadow_map); F(ChunkSet, shadow_map_length); F(ChunkSet, shadow_map_size);
	F(ChunkMD, mutex_read); F(ChunkMD, mutex_write); F(ChunkMD, readers); F(ChunkMD, last_access);
	F(ChunkMD, last_meshing); F(ChunkMD, count); F(ChunkMD, offset); F(ChunkMD, voxels); F(ChunkMD, rle);
	F(ChunkMD, mutex_svl); F(ChunkMD, dirty); F(ChunkMD, changing); F(ChunkMD, remesh); F(ChunkMD, make_mesh);
	F(ChunkMD, svl_dirty); F(ChunkMD, mesh_dirty); F(ChunkMD, no_geometry); F(ChunkMD, mesh_has_vbo);
	F(ChunkMD, svl); F(ChunkMD, svl_items); F(ChunkMD, svl_items_total); F(ChunkMD, mesh_vbo);
	F(ChunkMD, mesh_vbo_items); F(ChunkMD, mesh_ibo); F(ChunkMD, mesh_ibo_items);
	return 0;
}
