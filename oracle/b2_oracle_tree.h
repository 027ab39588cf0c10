/*
 * Oracle dynamic AABB tree and broadphase — TEST INFRASTRUCTURE ONLY (the checker).
 *
 * CPU restatement of box2d-rs 0.0.4:
 *   B2dynamicTree  src/private/collision/b2_dynamic_tree.rs:6-489 (allocate/free node,
 *                  create/destroy/move proxy, insert_leaf, remove_leaf, balance),
 *                  query src/b2_dynamic_tree.rs:239-267
 *   B2broadPhase   src/private/collision/b2_broad_phase.rs:33-111,
 *                  update_pairs src/b2_broad_phase.rs:200-249
 * Proxy ids are node-pool indices exactly as in the reference, so the
 * min/max proxy-id ordering of emitted pairs is reproduced.
 */
#ifndef B2_ORACLE_TREE_H
#define B2_ORACLE_TREE_H

#include <cmath>
#include <vector>
#include "b2_oracle_math.h"

namespace ora {

constexpr int kNullNode = -1;

struct TreeNode {
    AABB aabb{};
    int user = -1;      /* fixture index for leaves */
    int parent = kNullNode;  /* doubles as "next" in the free list */
    int child1 = kNullNode, child2 = kNullNode;
    int height = -1;
    bool moved = false;
    bool is_leaf() const { return child1 == kNullNode; }
};

class DynamicTree {
   public:
    DynamicTree();
    int create_proxy(const AABB& aabb, int user);
    /* state import: insert a leaf whose fat AABB is given as is, not marked moved */
    int create_proxy_fat(const AABB& fat, int user);
    void destroy_proxy(int id);
    bool move_proxy(int id, const AABB& aabb, Vec2 displacement);
    const AABB& fat_aabb(int id) const { return nodes_[id].aabb; }
    int user(int id) const { return nodes_[id].user; }
    bool was_moved(int id) const { return nodes_[id].moved; }
    void clear_moved(int id) { nodes_[id].moved = false; }
    int height() const { return root_ == kNullNode ? 0 : nodes_[root_].height; }
    template <class F>
    void query(const AABB& aabb, F&& cb) const {
        stack_.clear();
        stack_.push_back(root_);
        while (!stack_.empty()) {
            int id = stack_.back();
            stack_.pop_back();
            if (id == kNullNode) continue;
            const TreeNode& n = nodes_[id];
            if (overlap(n.aabb, aabb)) {
                if (n.is_leaf()) {
                    if (!cb(id)) return;
                } else {
                    stack_.push_back(n.child1);
                    stack_.push_back(n.child2);
                }
            }
        }
    }

    /* ray_cast, src/b2_dynamic_tree.rs:269-347: cb(max_fraction, proxy) returns the client's
     * value: 0 stops the cast, a positive value clips the segment to that fraction */
    template <class F>
    void ray_cast(Vec2 p1, Vec2 p2, float max_fraction, F&& cb) const {
        Vec2 r = p2 - p1;
        normalize(r);
        const Vec2 v = Vec2{-1.0f * r.y, 1.0f * r.x};  /* b2_cross_scalar_by_vec(1, r) */
        const Vec2 abs_v = Vec2{std::fabs(v.x), std::fabs(v.y)};
        AABB seg;
        {
            const Vec2 t = p1 + max_fraction * (p2 - p1);
            seg.lo = vmin(p1, t);
            seg.hi = vmax(p1, t);
        }
        stack_.clear();
        stack_.push_back(root_);
        while (!stack_.empty()) {
            const int id = stack_.back();
            stack_.pop_back();
            if (id == kNullNode) continue;
            const TreeNode& n = nodes_[id];
            if (!overlap(n.aabb, seg)) continue;
            const Vec2 c = 0.5f * (n.aabb.lo + n.aabb.hi);
            const Vec2 h = 0.5f * (n.aabb.hi - n.aabb.lo);
            const float separation = std::fabs(dot(v, p1 - c)) - dot(abs_v, h);
            if (separation > 0.0f) continue;
            if (n.is_leaf()) {
                const float value = cb(max_fraction, id);
                if (value == 0.0f) return;
                if (value > 0.0f) {
                    max_fraction = value;
                    const Vec2 t = p1 + max_fraction * (p2 - p1);
                    seg.lo = vmin(p1, t);
                    seg.hi = vmax(p1, t);
                }
            } else {
                stack_.push_back(n.child1);
                stack_.push_back(n.child2);
            }
        }
    }

   private:
    int allocate_node();
    void free_node(int id);
    void insert_leaf(int leaf);
    void remove_leaf(int leaf);
    int balance(int iA);

    std::vector<TreeNode> nodes_;
    int root_ = kNullNode;
    int node_count_ = 0;
    int free_list_ = 0;
    mutable std::vector<int> stack_;
};

struct Pair {
    int a, b;  /* proxy ids, a = min, b = max */
};

class BroadPhase {
   public:
    int create_proxy(const AABB& aabb, int user);
    int create_proxy_fat(const AABB& fat, int user) {
        ++proxy_count;
        return tree.create_proxy_fat(fat, user);
    }
    void destroy_proxy(int id);
    void move_proxy(int id, const AABB& aabb, Vec2 displacement);
    void touch_proxy(int id) { buffer_move(id); }
    bool test_overlap(int a, int b) const { return overlap(tree.fat_aabb(a), tree.fat_aabb(b)); }
    /* Fills `pairs` per update_pairs, clears moved flags and the move buffer. */
    void update_pairs(std::vector<Pair>& pairs);
    const std::vector<int>& move_buffer() const { return move_buffer_; }
    DynamicTree tree;
    int proxy_count = 0;

   private:
    void buffer_move(int id) { move_buffer_.push_back(id); }
    std::vector<int> move_buffer_;
};

}  // namespace ora
#endif
