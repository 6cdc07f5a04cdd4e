// tree.hpp -- dated binary tree with the reference's dirty tracking.
//
// Restates crates/b3/src/parameters/tree.rs for the native MCMC driver:
// node ids (leaves 0..L-1, internals L..2L-2, edge id = child id,
// tree.rs:728-736), mark_edge_updated (tree.rs:357-374), the children-first
// dirty list of partials_lists (tree.rs:398-461), the moves replace_child,
// set_height, set_root, swap_parents and scale (tree.rs:335-552), and
// accept/reject over epoch-backed arrays (tree.rs:975-994).
#pragma once

#include <cstdint>
#include <vector>

namespace b3g {

constexpr uint32_t kTombstone = 0xFFFFFFFFu;

class DatedTree {
      public:
	// parents[2L-1] (root: kTombstone) and heights[2L-1]; children are
	// filled in node order (load_parents, tree.rs:906-930).
	DatedTree(const uint32_t *parents, const double *heights,
		  uint32_t num_nodes);

	uint32_t num_leaves() const { return L_; }
	uint32_t num_internals() const { return L_ - 1; }
	uint32_t num_nodes() const { return 2 * L_ - 1; }
	uint32_t root() const { return root_; }
	bool is_leaf(uint32_t v) const { return v < L_; }
	double height(uint32_t v) const { return heights_[v]; }
	uint32_t parent_of(uint32_t v) const { return parents_[v]; }
	uint32_t left(uint32_t v) const { return children_[2 * (v - L_)]; }
	uint32_t right(uint32_t v) const { return children_[2 * (v - L_) + 1]; }
	uint32_t other_child(uint32_t parent, uint32_t child) const;
	double edge_length(uint32_t e) const
	{
		return heights_[parents_[e]] - heights_[e];
	}

	// dirty tracking
	void mark_edge_updated(uint32_t edge);
	void mark_all_edges_updated();
	bool is_changed() const { return any_edge_; }
	// Children-first dirty internals (root last), sorted child pairs and
	// the time lengths of both child edges.
	void partials_lists(std::vector<uint32_t> &internals,
			    std::vector<uint32_t> &children,
			    std::vector<double> &lengths) const;

	// moves (record old values for reject)
	void set_height(uint32_t node, double h);
	bool replace_child(uint32_t parent, uint32_t old_child,
			   uint32_t new_child);
	void set_root(uint32_t node);
	bool swap_parents(uint32_t a, uint32_t b);
	void scale(double factor);
	bool node_height_valid(uint32_t node) const;
	bool validate() const;

	void accept();
	void reject();

	// children[2 (v - L) + k], k = 0, 1: the order of every internal's
	// children (operators walk children in this order, so it is part of a
	// chain's state)
	const std::vector<uint32_t> &children() const { return children_; }
	// Sets that order; returns false, changing nothing, unless every
	// internal's pair is its two children under parents().
	bool set_child_order(const uint32_t *children);
	const std::vector<uint32_t> &parents() const { return parents_; }
	const std::vector<double> &heights() const { return heights_; }
	double root_height() const { return heights_[root_]; }

      private:
	void log_parent(uint32_t v);
	void log_child(uint32_t slot);
	void log_height(uint32_t v);
	void clear_updated();

	uint32_t L_;
	uint32_t root_, root_backup_;
	std::vector<uint32_t> parents_, children_;
	std::vector<double> heights_;
	// undo journals of the current epoch: (index, old value)
	std::vector<std::pair<uint32_t, uint32_t>> parent_log_, child_log_;
	std::vector<std::pair<uint32_t, double>> height_log_;
	std::vector<uint8_t> parent_logged_, child_logged_, height_logged_;
	// dirty bitmaps (tree.rs:46-50) and the nodes they mark
	std::vector<uint8_t> updated_edges_, updated_partials_;
	std::vector<uint32_t> marked_;
	bool any_edge_ = false;
	bool all_marked_ = false;
};

} // namespace b3g
