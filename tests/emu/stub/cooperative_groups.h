// Stand-in for cooperative_groups in the host emulation of the kernels: the
// cluster calls go to the emulation program (rank of this CTA, cluster barrier,
// the address of a word in a peer CTA's shared memory).
#pragma once
int emu_cta_rank();
void emu_cluster_sync();
void *emu_map_shared(void *p, int rank);
namespace cooperative_groups {
struct cluster_group {
	unsigned block_rank() const { return (unsigned)emu_cta_rank(); }
	void sync() { emu_cluster_sync(); }
	template <class T> T *map_shared_rank(T *p, int r) { return (T *)emu_map_shared((void *)p, r); }
};
inline cluster_group this_cluster() { return {}; }
}
