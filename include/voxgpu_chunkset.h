/*
 * voxgpu_chunkset.h — binary layout of the reference's chunk-set types
 * (kosshi-net/voxplat src/chunkset.h:9-118), for callers of the drop-in
 * entry points (voxgpu_dropin.h) that do not compile against the reference
 * headers. A program that already includes the reference's chunkset.h uses
 * those definitions instead: this header defines nothing once CHUNKSET_H is
 * set, and the drop-in library reads exactly these fields in this order.
 */
#ifndef VOXGPU_CHUNKSET_H
#define VOXGPU_CHUNKSET_H

#ifndef CHUNKSET_H
#include <pthread.h>
#include <stdint.h>

typedef uint8_t Voxel;

#define MAX_LOD_LEVEL 5

struct GeometrySVL {
	uint8_t lod;
	uint32_t vao;
	uint32_t vbo;
	uint32_t vbo_items;
};

struct GeometryMesh {
	uint32_t vao;
	uint32_t vbo;
	uint32_t vbo_items;
	uint32_t ibo;
	uint32_t ibo_items;
};

struct ChunkSet {
	uint32_t count;            /* chunks in the set */
	uint32_t chunk_count;
	uint32_t voxel_count;
	uint16_t root;             /* chunk edge length, a power of two */
	uint8_t root_bitw;
	uint16_t max[3];           /* chunks per axis */
	uint8_t max_bitw[3];
	struct GeometrySVL *gsvl[MAX_LOD_LEVEL];
	struct GeometryMesh *gmesh;
	struct ChunkMD *chunks;
	struct ChunkMD *null_chunk; /* shared all-air chunk */
	uint16_t *shadow_map;
	uint32_t shadow_map_length;
	uint32_t shadow_map_size[2]; /* X + Y, Z */
};

struct ChunkMD {
	pthread_mutex_t mutex_read;
	pthread_mutex_t mutex_write;
	uint16_t readers;
	float last_access;
	float last_meshing;
	uint32_t count;
	uint16_t offset[3];        /* chunk coordinates */
	Voxel *voxels;             /* decoded voxels, or NULL */
	Voxel *rle;                /* RLE stream, or NULL */
	pthread_mutex_t mutex_svl;
	volatile uint8_t dirty;
	volatile uint8_t changing;
	volatile uint8_t remesh;
	volatile uint8_t make_mesh;
	volatile uint8_t svl_dirty;
	volatile uint8_t mesh_dirty;
	volatile uint8_t no_geometry;
	int8_t mesh_has_vbo;
	uint16_t *svl;             /* splat lists, LOD 0 first */
	uint32_t svl_items[MAX_LOD_LEVEL];
	uint32_t svl_items_total;
	void *mesh_vbo;
	uint32_t mesh_vbo_items;
	void *mesh_ibo;
	uint32_t mesh_ibo_items;
};
#endif /* CHUNKSET_H */

#endif
