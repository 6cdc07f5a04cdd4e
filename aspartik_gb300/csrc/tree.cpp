// tree.cpp -- DatedTree (see tree.hpp for the reference lines it restates).
#include "tree.hpp"

#include <algorithm>
#include <deque>
#include <stdexcept>

namespace b3g {

DatedTree::DatedTree(const uint32_t *parents, const double *heights,
		     uint32_t num_nodes)
{
	if (num_nodes < 3 || num_nodes % 2 == 0)
		throw std::invalid_argument("a binary tree has 2L-1 >= 3 nodes");
	L_ = (num_nodes + 1) / 2;
	parents_.assign(parents, parents + num_nodes);
	heights_.assign(heights, heights + num_nodes);
	children_.assign(2 * (L_ - 1), kTombstone);
	root_ = kTombstone;
	for (uint32_t v = 0; v < num_nodes; ++v) {
		const uint32_t p = parents_[v];
		if (p == kTombstone) {
			if (root_ != kTombstone)
				throw std::invalid_argument("more than one root");
			root_ = v;
			continue;
		}
		if (p < L_ || p >= num_nodes)
			throw std::invalid_argument("a parent is not an internal node");
		const uint32_t k = 2 * (p - L_);
		if (children_[k] == kTombstone)
			children_[k] = v;
		else if (children_[k + 1] == kTombstone)
			children_[k + 1] = v;
		else
			throw std::invalid_argument("an internal node has 3 children");
	}
	if (root_ == kTombstone || root_ < L_)
		throw std::invalid_argument("no internal root");
	root_backup_ = root_;
	parent_logged_.assign(num_nodes, 0);
	height_logged_.assign(num_nodes, 0);
	child_logged_.assign(children_.size(), 0);
	updated_edges_.assign(num_nodes, 0);
	updated_partials_.assign(num_nodes, 0);
	if (!validate())
		throw std::invalid_argument("invalid tree (heights or links)");
}

bool DatedTree::set_child_order(const uint32_t *children)
{
	for (uint32_t k = 0; k < children_.size(); k += 2) {
		const uint32_t a = children[k], b = children[k + 1];
		const uint32_t x = children_[k], y = children_[k + 1];
		if (!((a == x && b == y) || (a == y && b == x)))
			return false;
	}
	children_.assign(children, children + children_.size());
	return true;
}

uint32_t DatedTree::other_child(uint32_t parent, uint32_t child) const
{
	const uint32_t l = left(parent), r = right(parent);
	return child == l ? r : l;
}

// tree.rs:357-374: the edge, then every ancestor until one that is already
// marked
void DatedTree::mark_edge_updated(uint32_t edge)
{
	if (!updated_edges_[edge]) {
		updated_edges_[edge] = 1;
		marked_.push_back(edge);
	}
	any_edge_ = true;
	uint32_t curr = edge;
	while (parents_[curr] != kTombstone) {
		curr = parents_[curr];
		if (updated_partials_[curr])
			break;
		updated_partials_[curr] = 1;
		marked_.push_back(curr);
	}
}

// tree.rs:382-386
void DatedTree::mark_all_edges_updated()
{
	std::fill(updated_edges_.begin(), updated_edges_.end(), 1);
	std::fill(updated_partials_.begin(), updated_partials_.end(), 1);
	any_edge_ = true;
	all_marked_ = true;
}

// updated_internals + children_list (tree.rs:398-434): breadth-first from
// the root over marked internals, reversed; the root is always listed
void DatedTree::partials_lists(std::vector<uint32_t> &internals,
			       std::vector<uint32_t> &children,
			       std::vector<double> &lengths) const
{
	internals.clear();
	children.clear();
	lengths.clear();
	internals.push_back(root_);
	size_t head = 0;
	while (head < internals.size()) {
		const uint32_t v = internals[head++];
		for (const uint32_t ch : {left(v), right(v)})
			if (updated_partials_[ch] && ch >= L_)
				internals.push_back(ch);
	}
	std::reverse(internals.begin(), internals.end());
	for (const uint32_t v : internals) {
		uint32_t l = left(v), r = right(v);
		if (r < l)
			std::swap(l, r);
		children.push_back(l);
		children.push_back(r);
		lengths.push_back(heights_[v] - heights_[l]);
		lengths.push_back(heights_[v] - heights_[r]);
	}
}

void DatedTree::log_parent(uint32_t v)
{
	if (!parent_logged_[v]) {
		parent_logged_[v] = 1;
		parent_log_.emplace_back(v, parents_[v]);
	}
}

void DatedTree::log_child(uint32_t slot)
{
	if (!child_logged_[slot]) {
		child_logged_[slot] = 1;
		child_log_.emplace_back(slot, children_[slot]);
	}
}

void DatedTree::log_height(uint32_t v)
{
	if (!height_logged_[v]) {
		height_logged_[v] = 1;
		height_log_.emplace_back(v, heights_[v]);
	}
}

// tree.rs:516-527
void DatedTree::set_height(uint32_t node, double h)
{
	log_height(node);
	heights_[node] = h;
	if (parents_[node] != kTombstone)
		mark_edge_updated(node);
	if (node >= L_) {
		mark_edge_updated(left(node));
		mark_edge_updated(right(node));
	}
}

// tree.rs:471-495
bool DatedTree::replace_child(uint32_t parent, uint32_t old_child,
			      uint32_t new_child)
{
	const uint32_t k = 2 * (parent - L_);
	uint32_t slot;
	if (children_[k] == old_child)
		slot = k;
	else if (children_[k + 1] == old_child)
		slot = k + 1;
	else
		return false;
	log_parent(new_child);
	parents_[new_child] = parent;
	log_child(slot);
	children_[slot] = new_child;
	mark_edge_updated(new_child);
	return true;
}

// tree.rs:529-533
void DatedTree::set_root(uint32_t node)
{
	root_ = node;
	log_parent(node);
	parents_[node] = kTombstone;
}

// tree.rs:552-568
bool DatedTree::node_height_valid(uint32_t node) const
{
	const double h = heights_[node];
	if (parents_[node] != kTombstone && !(h < heights_[parents_[node]]))
		return false;
	if (node < L_)
		return true;
	return h > heights_[left(node)] && h > heights_[right(node)];
}

// tree.rs:535-550
bool DatedTree::swap_parents(uint32_t a, uint32_t b)
{
	const uint32_t pa = parents_[a], pb = parents_[b];
	if (pa == kTombstone || pb == kTombstone)
		return false;
	if (!replace_child(pa, a, b) || !replace_child(pb, b, a))
		return false;
	return node_height_valid(a) && node_height_valid(b);
}

// tree.rs:335-348 (all leaves here are contemporary)
void DatedTree::scale(double factor)
{
	for (uint32_t v = L_; v < num_nodes(); ++v)
		set_height(v, heights_[v] * factor);
}

// tree.rs:584-651 (the structural checks)
bool DatedTree::validate() const
{
	uint32_t roots = 0;
	for (uint32_t v = 0; v < num_nodes(); ++v) {
		if (parents_[v] == kTombstone) {
			++roots;
			if (v != root_)
				return false;
		} else if (parents_[v] < L_) {
			return false;
		}
	}
	if (roots != 1)
		return false;
	for (uint32_t v = L_; v < num_nodes(); ++v) {
		const uint32_t l = left(v), r = right(v);
		if (l == kTombstone || r == kTombstone || l == r)
			return false;
		if (parents_[l] != v || parents_[r] != v)
			return false;
		if (!(heights_[v] > heights_[l] && heights_[v] > heights_[r]))
			return false;
	}
	return true;
}

void DatedTree::clear_updated()
{
	if (all_marked_) {
		std::fill(updated_edges_.begin(), updated_edges_.end(), 0);
		std::fill(updated_partials_.begin(), updated_partials_.end(), 0);
	} else {
		for (const uint32_t v : marked_) {
			updated_edges_[v] = 0;
			updated_partials_[v] = 0;
		}
	}
	marked_.clear();
	all_marked_ = false;
	any_edge_ = false;
}

void DatedTree::accept()
{
	for (const auto &e : parent_log_)
		parent_logged_[e.first] = 0;
	for (const auto &e : child_log_)
		child_logged_[e.first] = 0;
	for (const auto &e : height_log_)
		height_logged_[e.first] = 0;
	parent_log_.clear();
	child_log_.clear();
	height_log_.clear();
	root_backup_ = root_;
	clear_updated();
}

void DatedTree::reject()
{
	for (auto it = parent_log_.rbegin(); it != parent_log_.rend(); ++it) {
		parents_[it->first] = it->second;
		parent_logged_[it->first] = 0;
	}
	for (auto it = child_log_.rbegin(); it != child_log_.rend(); ++it) {
		children_[it->first] = it->second;
		child_logged_[it->first] = 0;
	}
	for (auto it = height_log_.rbegin(); it != height_log_.rend(); ++it) {
		heights_[it->first] = it->second;
		height_logged_[it->first] = 0;
	}
	parent_log_.clear();
	child_log_.clear();
	height_log_.clear();
	root_ = root_backup_;
	clear_updated();
}

} // namespace b3g
