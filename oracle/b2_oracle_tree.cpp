/*
 * Oracle dynamic tree / broadphase — TEST INFRASTRUCTURE ONLY (the checker).
 * Reference lines are cited per function; compile with -ffp-contract=off.
 */
#include "b2_oracle_tree.h"

namespace ora {

/* b2_dynamic_tree(), private/collision/b2_dynamic_tree.rs:6-27 */
DynamicTree::DynamicTree() {
    nodes_.resize(16);
    for (int i = 0; i < 15; ++i) {
        nodes_[i].parent = i + 1;
        nodes_[i].height = -1;
    }
    nodes_[15].parent = kNullNode;
    nodes_[15].height = -1;
    free_list_ = 0;
    stack_.reserve(256);
}

/* allocate_node, :28-52 */
int DynamicTree::allocate_node() {
    if (free_list_ == kNullNode) {
        int cap = (int)nodes_.size();
        nodes_.resize((size_t)cap * 2);
        for (int i = node_count_; i < cap * 2 - 1; ++i) {
            nodes_[i].parent = i + 1;
            nodes_[i].height = -1;
        }
        nodes_[cap * 2 - 1].parent = kNullNode;
        nodes_[cap * 2 - 1].height = -1;
        free_list_ = node_count_;
    }
    int id = free_list_;
    free_list_ = nodes_[id].parent;
    TreeNode& n = nodes_[id];
    n.parent = kNullNode;
    n.child1 = kNullNode;
    n.child2 = kNullNode;
    n.height = 0;
    n.user = -1;
    n.moved = false;
    ++node_count_;
    return id;
}

/* free_node, :53-60 */
void DynamicTree::free_node(int id) {
    nodes_[id].parent = free_list_;
    nodes_[id].height = -1;
    free_list_ = id;
    --node_count_;
}

/* create_proxy, :61-76 */
int DynamicTree::create_proxy(const AABB& aabb, int user) {
    int id = allocate_node();
    Vec2 r{kAabbExtension, kAabbExtension};
    nodes_[id].aabb.lo = aabb.lo - r;
    nodes_[id].aabb.hi = aabb.hi + r;
    nodes_[id].user = user;
    nodes_[id].height = 0;
    nodes_[id].moved = true;
    insert_leaf(id);
    return id;
}

int DynamicTree::create_proxy_fat(const AABB& fat, int user) {
    int id = allocate_node();
    nodes_[id].aabb = fat;
    nodes_[id].user = user;
    nodes_[id].height = 0;
    nodes_[id].moved = false;
    insert_leaf(id);
    return id;
}

void DynamicTree::destroy_proxy(int id) {
    remove_leaf(id);
    free_node(id);
}

/* move_proxy, :109-168 */
bool DynamicTree::move_proxy(int id, const AABB& aabb, Vec2 displacement) {
    Vec2 r{kAabbExtension, kAabbExtension};
    AABB fat{aabb.lo - r, aabb.hi + r};
    Vec2 d = kAabbMultiplier * displacement;
    if (d.x < 0.0f) fat.lo.x += d.x; else fat.hi.x += d.x;
    if (d.y < 0.0f) fat.lo.y += d.y; else fat.hi.y += d.y;
    const AABB treeAabb = nodes_[id].aabb;
    if (contains(treeAabb, aabb)) {
        AABB huge{fat.lo - 4.0f * r, fat.hi + 4.0f * r};
        if (contains(huge, treeAabb)) return false;
    }
    remove_leaf(id);
    nodes_[id].aabb = fat;
    insert_leaf(id);
    nodes_[id].moved = true;
    return true;
}

/* insert_leaf, :170-298 (perimeter cost descent, then balance walking up) */
void DynamicTree::insert_leaf(int leaf) {
    if (root_ == kNullNode) {
        root_ = leaf;
        nodes_[root_].parent = kNullNode;
        return;
    }
    const AABB leafAabb = nodes_[leaf].aabb;
    int index = root_;
    while (!nodes_[index].is_leaf()) {
        int c1 = nodes_[index].child1;
        int c2 = nodes_[index].child2;
        float area = perimeter(nodes_[index].aabb);
        AABB combined = combine(nodes_[index].aabb, leafAabb);
        float combinedArea = perimeter(combined);
        float cost = 2.0f * combinedArea;
        float inheritance = 2.0f * (combinedArea - area);
        float cost1, cost2;
        {
            AABB a = combine(leafAabb, nodes_[c1].aabb);
            if (nodes_[c1].is_leaf()) cost1 = perimeter(a) + inheritance;
            else cost1 = (perimeter(a) - perimeter(nodes_[c1].aabb)) + inheritance;
        }
        {
            AABB a = combine(leafAabb, nodes_[c2].aabb);
            if (nodes_[c2].is_leaf()) cost2 = perimeter(a) + inheritance;
            else cost2 = perimeter(a) - perimeter(nodes_[c2].aabb) + inheritance;
        }
        if (cost < cost1 && cost < cost2) break;
        index = (cost1 < cost2) ? c1 : c2;
    }
    int sibling = index;
    int oldParent = nodes_[sibling].parent;
    int newParent = allocate_node();
    nodes_[newParent].parent = oldParent;
    nodes_[newParent].user = -1;
    nodes_[newParent].aabb = combine(leafAabb, nodes_[sibling].aabb);
    nodes_[newParent].height = nodes_[sibling].height + 1;
    if (oldParent != kNullNode) {
        if (nodes_[oldParent].child1 == sibling) nodes_[oldParent].child1 = newParent;
        else nodes_[oldParent].child2 = newParent;
    } else {
        root_ = newParent;
    }
    nodes_[newParent].child1 = sibling;
    nodes_[newParent].child2 = leaf;
    nodes_[sibling].parent = newParent;
    nodes_[leaf].parent = newParent;
    index = nodes_[leaf].parent;
    while (index != kNullNode) {
        index = balance(index);
        int c1 = nodes_[index].child1;
        int c2 = nodes_[index].child2;
        nodes_[index].height = 1 + bmax(nodes_[c1].height, nodes_[c2].height);
        nodes_[index].aabb = combine(nodes_[c1].aabb, nodes_[c2].aabb);
        index = nodes_[index].parent;
    }
}

/* remove_leaf, :300-353 */
void DynamicTree::remove_leaf(int leaf) {
    if (leaf == root_) {
        root_ = kNullNode;
        return;
    }
    int parent = nodes_[leaf].parent;
    int grand = nodes_[parent].parent;
    int sibling = (nodes_[parent].child1 == leaf) ? nodes_[parent].child2 : nodes_[parent].child1;
    if (grand != kNullNode) {
        if (nodes_[grand].child1 == parent) nodes_[grand].child1 = sibling;
        else nodes_[grand].child2 = sibling;
        nodes_[sibling].parent = grand;
        free_node(parent);
        int index = grand;
        while (index != kNullNode) {
            index = balance(index);
            int c1 = nodes_[index].child1;
            int c2 = nodes_[index].child2;
            nodes_[index].aabb = combine(nodes_[c1].aabb, nodes_[c2].aabb);
            nodes_[index].height = 1 + bmax(nodes_[c1].height, nodes_[c2].height);
            index = nodes_[index].parent;
        }
    } else {
        root_ = sibling;
        nodes_[sibling].parent = kNullNode;
        free_node(parent);
    }
}

/* balance (AVL-style rotation of A with its taller child), :357-489 */
int DynamicTree::balance(int iA) {
    TreeNode* A = &nodes_[iA];
    if (A->is_leaf() || A->height < 2) return iA;
    int iB = A->child1, iC = A->child2;
    TreeNode* B = &nodes_[iB];
    TreeNode* C = &nodes_[iC];
    int bal = C->height - B->height;
    if (bal > 1) {  /* rotate C up */
        int iF = C->child1, iG = C->child2;
        TreeNode* F = &nodes_[iF];
        TreeNode* G = &nodes_[iG];
        C->child1 = iA;
        C->parent = A->parent;
        A->parent = iC;
        if (C->parent != kNullNode) {
            if (nodes_[C->parent].child1 == iA) nodes_[C->parent].child1 = iC;
            else nodes_[C->parent].child2 = iC;
        } else {
            root_ = iC;
        }
        if (F->height > G->height) {
            C->child2 = iF;
            A->child2 = iG;
            G->parent = iA;
            A->aabb = combine(B->aabb, G->aabb);
            C->aabb = combine(A->aabb, F->aabb);
            A->height = 1 + bmax(B->height, G->height);
            C->height = 1 + bmax(A->height, F->height);
        } else {
            C->child2 = iG;
            A->child2 = iF;
            F->parent = iA;
            A->aabb = combine(B->aabb, F->aabb);
            C->aabb = combine(A->aabb, G->aabb);
            A->height = 1 + bmax(B->height, F->height);
            C->height = 1 + bmax(A->height, G->height);
        }
        return iC;
    }
    if (bal < -1) {  /* rotate B up */
        int iD = B->child1, iE = B->child2;
        TreeNode* D = &nodes_[iD];
        TreeNode* E = &nodes_[iE];
        B->child1 = iA;
        B->parent = A->parent;
        A->parent = iB;
        if (B->parent != kNullNode) {
            if (nodes_[B->parent].child1 == iA) nodes_[B->parent].child1 = iB;
            else nodes_[B->parent].child2 = iB;
        } else {
            root_ = iB;
        }
        if (D->height > E->height) {
            B->child2 = iD;
            A->child1 = iE;
            E->parent = iA;
            A->aabb = combine(C->aabb, E->aabb);
            B->aabb = combine(A->aabb, D->aabb);
            A->height = 1 + bmax(C->height, E->height);
            B->height = 1 + bmax(A->height, D->height);
        } else {
            B->child2 = iE;
            A->child1 = iD;
            D->parent = iA;
            A->aabb = combine(C->aabb, D->aabb);
            B->aabb = combine(A->aabb, E->aabb);
            A->height = 1 + bmax(C->height, D->height);
            B->height = 1 + bmax(A->height, E->height);
        }
        return iB;
    }
    return iA;
}

/* b2_broad_phase_create_proxy / destroy / move, private/collision/b2_broad_phase.rs:33-60 */
int BroadPhase::create_proxy(const AABB& aabb, int user) {
    int id = tree.create_proxy(aabb, user);
    ++proxy_count;
    buffer_move(id);
    return id;
}

void BroadPhase::destroy_proxy(int id) {
    for (int& m : move_buffer_)
        if (m == id) m = kNullNode;
    --proxy_count;
    tree.destroy_proxy(id);
}

void BroadPhase::move_proxy(int id, const AABB& aabb, Vec2 displacement) {
    if (tree.move_proxy(id, aabb, displacement)) buffer_move(id);
}

/* update_pairs, src/b2_broad_phase.rs:200-249 with the query callback of
 * private/collision/b2_broad_phase.rs:86-111 */
void BroadPhase::update_pairs(std::vector<Pair>& pairs) {
    pairs.clear();
    for (int q : move_buffer_) {
        if (q == kNullNode) continue;
        const AABB fat = tree.fat_aabb(q);
        tree.query(fat, [&](int id) {
            if (id == q) return true;
            if (tree.was_moved(id) && id > q) return true;
            pairs.push_back(Pair{bmin(id, q), bmax(id, q)});
            return true;
        });
    }
    for (int q : move_buffer_)
        if (q != kNullNode) tree.clear_moved(q);
    move_buffer_.clear();
}

}  // namespace ora
