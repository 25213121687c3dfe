// Stand-in for cooperative_groups: the grid kernel's headers name cluster
// groups, the grid path never uses them (a call aborts the emulation).
#pragma once
#include <cstdlib>
namespace cooperative_groups {
struct cluster_group {
	unsigned block_rank() const { abort(); }
	void sync() { abort(); }
	template <class T> T *map_shared_rank(T *, int) { abort(); }
};
inline cluster_group this_cluster() { return {}; }
}
