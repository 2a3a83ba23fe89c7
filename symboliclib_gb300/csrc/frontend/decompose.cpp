// Decomposition of expression DAGs into reusable blocks.
//
// Restates the method of reference src/Decomposition.cpp:234-490: sub-trees of
// sufficient complexity that occur more than once (by node identity) become
// blocks; small blocks are merged into their parents, single-parent blocks are
// inlined, levels are assigned from the outputs down, and each surviving block
// is re-expressed with its child blocks replaced by variables of
// `variableGroupId`.  Orders (pre-order discovery, hash-ordered child maps,
// pointer-ordered reachable set, structure-hash sort of commutative operands)
// follow the reference because they determine the kernel templates.
#include <algorithm>
#include <map>
#include <set>
#include <unordered_map>

#include "symgb/stage_clock.hpp"
#include "symgb/frontend.hpp"
#include "symgb/parallel.hpp"
#include "symgb/traverse.hpp"

namespace symgb {

namespace {

constexpr unsigned char MERGED = 1;
constexpr unsigned char EXPLICITLY_MERGED = 2;
constexpr unsigned char FIXED_NODE = 3;

// Sort of a short range by a key; pairs are swapped directly and longer ranges
// use std::sort (reference src/Utilities.hpp:135-152).
template <class It, class Key>
void sortByKey(It first, It last, Key key) {
    const auto d = std::distance(first, last);
    if (d < 2) return;
    if (d == 2) {
        if (key(*first) > key(*(first + 1))) std::iter_swap(first, first + 1);
        return;
    }
    std::sort(first, last, [&](const auto& a, const auto& b) { return key(a) < key(b); });
}

struct Node {
    Symbolic x;  // extracted expression, once computed
    int id;
    Symbolic fullx;
    unsigned char status = 0;
    unsigned level = (unsigned)-1;
    unsigned char complexity = 0;
    hash_t structureHash = 0;
    unsigned numParents = 0;
    std::map<hash_t, Node*> childs;  // keyed by algebraic hash

    Node(const Symbolic& full, int id_) : id(id_), fullx(full) {}

    hash_t hash() const { return fullx.algebraicHash(); }

    void addChild(const std::pair<hash_t, Node*>& c) {
        if (childs.insert(c).second) ++c.second->numParents;
    }

    // Ids of all non-merged descendants reached through merged nodes.
    std::vector<int> allChildren() {
        std::vector<int> ret;
        std::vector<Node*> stack{this};
        while (!stack.empty()) {
            Node* cur = stack.back();
            stack.pop_back();
            for (auto& c : cur->childs) {
                if (c.second->status == MERGED)
                    stack.push_back(c.second);
                else
                    ret.push_back(c.second->id);
            }
        }
        std::sort(ret.begin(), ret.end());
        ret.erase(std::unique(ret.begin(), ret.end()), ret.end());
        return ret;
    }

    // Absorbs child `n` into this node's computation; n's children become ours.
    void merge(Node& n) {
        childs.erase(n.hash());
        if (n.status != EXPLICITLY_MERGED) {
            for (auto& c : n.childs) --c.second->numParents;
            n.numParents = 0;
            n.status = EXPLICITLY_MERGED;
        }
        for (auto& c : n.childs) addChild(c);
        complexity = (unsigned char)std::min(255, complexity + n.complexity);
    }

    // Merged children extracted during one top-level extraction, shared within
    // it (the same handle wherever the child occurs).
    using MergedMemo = std::unordered_map<const Node*, std::pair<Symbolic, hash_t>>;

    // This node's expression with non-merged child nodes replaced by
    // variables of `groupId` and merged children inlined, and its structure
    // hash.  Reads the node graph only, so blocks can be extracted in parallel.
    std::pair<Symbolic, hash_t> extract(int groupId, MergedMemo& merged) const {
        std::vector<std::pair<Symbolic, hash_t>> stack;
        KeyMap<std::pair<Symbolic, hash_t>> cache;

        auto pre = [&](const Symbolic& y) {
            if (auto* itc = cache.find(y.id())) {
                stack.push_back(*itc);
                return false;
            }
            if (y.op() == FIXED) {
                stack.emplace_back(y[0], VarHash);
                return false;
            }
            auto it = childs.find(y.ahash());
            if (it != childs.end()) {
                if (it->second->status == MERGED) {
                    auto m = merged.find(it->second);
                    if (m == merged.end()) {
                        auto r = it->second->extract(groupId, merged);
                        m = merged.emplace(it->second, std::move(r)).first;
                    }
                    stack.push_back(m->second);
                } else {
                    stack.emplace_back(Symbolic(it->second->id, groupId), VarHash);
                }
                return false;
            }
            return true;
        };

        auto post = [&](const Symbolic& y) {
            const unsigned nc = y.numChilds();
            if (nc == 0) {
                stack.emplace_back(y, y.op() == VAR ? VarHash : ConstHash);
                return;
            }
            if (opInfo(y.op()).commutative)
                sortByKey(stack.end() - nc, stack.end(), [](const auto& p) { return p.second; });
            std::vector<hash_t> hashes;
            hashes.reserve(nc + 1);
            Symbolic* kids = Symbolic::childArray(nc);
            Symbolic* out = kids;
            for (std::size_t i = stack.size() - nc; i < stack.size(); ++i) {
                *out++ = std::move(stack[i].first);
                hashes.push_back(stack[i].second);
            }
            hashes.push_back(opInfo(y.op()).seed);
            stack.erase(stack.end() - nc, stack.end());
            stack.emplace_back(Symbolic(y.op(), kids, nc), hashVector(hashes));
            cache[y.id()] = stack.back();
        };

        prePostOrderTraverse(fullx, pre, post);
        assert(stack.size() == 1);
        return stack.front();
    }

    // Fills x (wrapped as ASSIGN to this node's variable) and structureHash.
    void extractExpression(int groupId, MergedMemo& merged) {
        auto r = extract(groupId, merged);
        x = r.first;
        structureHash = r.second;
        if (x.op() != BLOCK && x.op() != ASSIGN && status != MERGED) x = Symbolic(ASSIGN, Symbolic(id, groupId), x);
    }
};

}  // namespace

std::vector<ExpressionBlock> decompose(const std::vector<Symbolic>& expr, unsigned char threshold, int groupId,
                                       bool mergeSingleParent) {
    if (threshold == 255) {  // decomposition disabled
        std::vector<ExpressionBlock> ret(expr.size());
        for (std::size_t i = 0; i < expr.size(); ++i) {
            ret[i].x = expr[i];
            ret[i].structureHash = expr[i].computeStructureHash();
        }
        return ret;
    }

    StageClock clock;
    std::vector<Node> nodes;
    nodes.reserve(5 * expr.size());
    // node identity -> (occurrence count, node index + 1)
    KeyMap<std::pair<unsigned, unsigned>> count(4 * expr.size());
    int id = 0;

    // 1. Count occurrences; a complex sub-expression seen twice becomes a node.
    for (const auto& x : expr) {
        preOrderTraverse(x, [&](const Symbolic& y) {
            if (y.op() == FIXED) {
                auto& xc = count[y[1].id()];
                if (xc.first++ == 0) {
                    nodes.emplace_back(y[1], id++);
                    nodes.back().status = FIXED_NODE;
                    xc.second = (unsigned)nodes.size();
                }
                return false;
            }
            if (y.complexity() < threshold) return false;
            auto& xc = count[y.id()];
            if (xc.first == 1) {
                nodes.emplace_back(y, id++);
                xc.second = (unsigned)nodes.size();
            }
            return xc.first++ == 0;
        });
    }

    clock.mark("decompose: count");

    // 2. One node per output expression.
    std::vector<unsigned> outputNodes;
    for (const auto& x : expr) {
        nodes.emplace_back(x, id++);
        nodes.back().numParents++;
        outputNodes.push_back((unsigned)nodes.size() - 1);
        count[x.id()].second = (unsigned)nodes.size();
    }

    // 3. Child links and node complexities.  Each node only reads the
    // occurrence map and the expression graph and writes its own links, so the
    // nodes are processed in parallel; parent counts are added afterwards.
    parallelFor(nodes.size(), 64, [&](std::size_t b, std::size_t e) {
        for (std::size_t ni = b; ni < e; ++ni) {
            Node& node = nodes[ni];
            if (node.status == FIXED_NODE) {
                node.complexity = 255;
                continue;
            }
            int comp = 0;
            preOrderTraverse(node.fullx, [&](const Symbolic& y) {
                if (y.op() == FIXED) {
                    const auto* d = count.find(y[1].id());
                    node.childs.insert({y[1].ahash(), nodes.data() + d->second - 1});
                    return false;
                }
                if (y.complexity() < threshold) {
                    comp += y.complexity();
                    return false;
                }
                const auto* d = count.find(y.id());
                if (d && d->second != 0 && y.ahash() != node.hash()) {
                    node.childs.insert({y.ahash(), nodes.data() + d->second - 1});
                    return false;
                }
                comp += std::max(1, (int)y.numChilds()) * opInfo(y.op()).cost;
                return true;
            });
            node.complexity = (unsigned char)std::min(255, comp);
        }
    });
    for (auto& node : nodes)
        for (auto& c : node.childs) ++c.second->numParents;
    clock.mark("decompose: links");

    // 4. Merge small and single-parent children, assign levels.  `reachable`
    // is a flag per node; nodes live in one array, so index order is the
    // pointer order of the reference's std::set<ExpressionNode*>.
    std::vector<Node*> stack;
    std::vector<char> reachable(nodes.size(), 0);
    auto insertReachable = [&](Node* n) {
        char& f = reachable[n - nodes.data()];
        const bool fresh = !f;
        f = 1;
        return fresh;
    };
    std::vector<Node*> childStack;
    for (unsigned i : outputNodes) {
        Node* x = nodes.data() + i;
        stack.clear();
        stack.push_back(x);
        x->level = 0;
        while (!stack.empty()) {
            Node* node = stack.back();
            stack.pop_back();
            if (node->status == FIXED_NODE) {
                insertReachable(node);
            } else if (node->status != 0 || insertReachable(node)) {
                childStack.clear();
                for (auto& c : node->childs) childStack.push_back(c.second);
                while (!childStack.empty()) {
                    Node* cn = childStack.back();
                    childStack.pop_back();
                    if (cn->status == FIXED_NODE) {
                    } else if (cn->status == EXPLICITLY_MERGED || cn->complexity < threshold) {
                        node->merge(*cn);
                        for (auto& c : cn->childs) childStack.push_back(c.second);
                    } else if (mergeSingleParent && cn->numParents == 1) {
                        cn->status = MERGED;
                        for (auto& c : cn->childs) stack.push_back(c.second);
                    }
                }
                for (auto& c : node->childs) {
                    c.second->level = node->level + 1;
                    stack.push_back(c.second);
                }
            }
        }
    }

    clock.mark("decompose: merge, levels");

    // 5. Blocks of the reachable, non-inlined nodes in node order.  Each
    // block's extraction only reads the node graph, so blocks are extracted
    // in parallel (reference counts atomic meanwhile).
    std::vector<int> blockIdMap(nodes.size(), -1);
    std::vector<std::size_t> blockNode;
    for (std::size_t ni = 0; ni < nodes.size(); ++ni) {
        if (!reachable[ni] || nodes[ni].status == MERGED) continue;
        blockIdMap[nodes[ni].id] = (int)blockNode.size();
        blockNode.push_back(ni);
    }
    std::vector<ExpressionBlock> blocks(blockNode.size());
    {
        Symbolic::ConcurrentRefs concurrent;
        parallelFor(blockNode.size(), 256, [&](std::size_t b, std::size_t e) {
            Node::MergedMemo merged;
            for (std::size_t i = b; i < e; ++i) {
                Node* x = &nodes[blockNode[i]];
                merged.clear();
                x->extractExpression(groupId, merged);
                blocks[i].level = (int)x->level;
                blocks[i].x = x->x;
                blocks[i].structureHash = x->structureHash;
                blocks[i].childs = x->allChildren();
            }
        });
    }
    for (auto& b : blocks)
        for (auto& c : b.childs) c = blockIdMap[c];
    clock.mark("decompose: extract");
    return blocks;
}

}  // namespace symgb
