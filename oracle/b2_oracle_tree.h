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
