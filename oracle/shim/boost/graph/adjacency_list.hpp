// Stand-in for the part of Boost.Graph that the reference's weave and its
// half-edge diagram use (adjacency_list with list storage, bidirectional),
// so the reference's weave, Waterline and AdaptiveWaterline sources compile
// unmodified into the oracle library (oracle/_ref).  Project-written; only
// the behaviour those sources rely on is provided:
//   - vertices and edges are heap nodes, their descriptors opaque pointers
//     (ordered by address, as Boost's list-storage descriptors are);
//   - vertices(g) and edges(g) iterate in insertion order, out_edges(v, g)
//     in the order the edges were added at v;
//   - parallel edges are allowed (add_edge always succeeds);
//   - removing an edge or a vertex frees it; clear_vertex removes every
//     edge in or out of the vertex.
#pragma once
#include <cstddef>
#include <functional>
#include <iostream>
#include <iterator>
#include <list>
#include <set>
#include <tuple>
#include <utility>
#include <vector>

namespace boost {

struct listS {};
struct vecS {};
struct setS {};
struct bidirectionalS {};
struct directedS {};
struct undirectedS {};
struct no_property {};

// Descriptor of a vertex or an edge: the address of its node.
template <int TAG>
struct graph_desc {
    void* p = nullptr;
    graph_desc() = default;
    explicit graph_desc(void* q) : p(q) {}
    friend bool operator==(graph_desc a, graph_desc b) { return a.p == b.p; }
    friend bool operator!=(graph_desc a, graph_desc b) { return a.p != b.p; }
    friend bool operator<(graph_desc a, graph_desc b) { return std::less<void*>()(a.p, b.p); }
    friend std::ostream& operator<<(std::ostream& o, graph_desc a) { return o << a.p; }
};
typedef graph_desc<0> shim_vertex_descriptor;
typedef graph_desc<1> shim_edge_descriptor;

template <class A = void, class B = void, class C = void, class D = void>
struct adjacency_list_traits {
    typedef shim_vertex_descriptor vertex_descriptor;
    typedef shim_edge_descriptor edge_descriptor;
};

// An iterator over a std::list of node pointers that yields descriptors.
template <class Node, class Desc>
class node_iterator {
   public:
    typedef std::bidirectional_iterator_tag iterator_category;
    typedef Desc value_type;
    typedef std::ptrdiff_t difference_type;
    typedef const Desc* pointer;
    typedef Desc reference;
    node_iterator() = default;
    explicit node_iterator(typename std::list<Node*>::const_iterator i) : it(i) {}
    Desc operator*() const { return Desc(*it); }
    node_iterator& operator++() { ++it; return *this; }
    node_iterator operator++(int) { node_iterator t = *this; ++it; return t; }
    node_iterator& operator--() { --it; return *this; }
    bool operator==(const node_iterator& o) const { return it == o.it; }
    bool operator!=(const node_iterator& o) const { return it != o.it; }
   private:
    typename std::list<Node*>::const_iterator it;
};

template <class OEL = vecS, class VL = vecS, class DIR = directedS, class VP = no_property,
          class EP = no_property, class GP = no_property, class EL = listS>
class adjacency_list {
   public:
    struct enode;
    struct vnode {
        VP prop;
        std::list<enode*> out, in;
        typename std::list<vnode*>::iterator at;  // position in vlist
    };
    struct enode {
        EP prop;
        vnode* s;
        vnode* t;
        typename std::list<enode*>::iterator at, at_out, at_in;  // positions in elist, s->out, t->in
    };
    typedef shim_vertex_descriptor vertex_descriptor;
    typedef shim_edge_descriptor edge_descriptor;
    typedef node_iterator<vnode, vertex_descriptor> vertex_iterator;
    typedef node_iterator<enode, edge_descriptor> edge_iterator;
    typedef node_iterator<enode, edge_descriptor> out_edge_iterator;
    typedef node_iterator<enode, edge_descriptor> in_edge_iterator;
    typedef node_iterator<vnode, vertex_descriptor> adjacency_iterator;
    typedef std::size_t vertices_size_type;
    typedef std::size_t edges_size_type;
    typedef std::size_t degree_size_type;

    adjacency_list() = default;
    adjacency_list(const adjacency_list&) = delete;
    adjacency_list& operator=(const adjacency_list&) = delete;
    ~adjacency_list() {
        for (enode* e : elist) delete e;
        for (vnode* v : vlist) delete v;
    }
    static vertex_descriptor null_vertex() { return vertex_descriptor(); }
    VP& operator[](vertex_descriptor v) { return static_cast<vnode*>(v.p)->prop; }
    const VP& operator[](vertex_descriptor v) const { return static_cast<const vnode*>(v.p)->prop; }
    EP& operator[](edge_descriptor e) { return static_cast<enode*>(e.p)->prop; }
    const EP& operator[](edge_descriptor e) const { return static_cast<const enode*>(e.p)->prop; }

    std::list<vnode*> vlist;
    std::list<enode*> elist;
};

template <class G>
struct graph_traits {
    typedef typename G::vertex_descriptor vertex_descriptor;
    typedef typename G::edge_descriptor edge_descriptor;
    typedef typename G::vertex_iterator vertex_iterator;
    typedef typename G::edge_iterator edge_iterator;
    typedef typename G::out_edge_iterator out_edge_iterator;
    typedef typename G::in_edge_iterator in_edge_iterator;
    typedef typename G::adjacency_iterator adjacency_iterator;
    typedef typename G::vertices_size_type vertices_size_type;
    typedef typename G::edges_size_type edges_size_type;
    typedef typename G::degree_size_type degree_size_type;
    static vertex_descriptor null_vertex() { return vertex_descriptor(); }
};

#define BOOST_SHIM_G adjacency_list<OEL, VL, DIR, VP, EP, GP, EL>
#define BOOST_SHIM_T template <class OEL, class VL, class DIR, class VP, class EP, class GP, class EL>

BOOST_SHIM_T shim_vertex_descriptor add_vertex(const VP& p, BOOST_SHIM_G& g) {
    auto* v = new typename BOOST_SHIM_G::vnode();
    v->prop = p;
    v->at = g.vlist.insert(g.vlist.end(), v);
    return shim_vertex_descriptor(v);
}
BOOST_SHIM_T shim_vertex_descriptor add_vertex(BOOST_SHIM_G& g) { return add_vertex(VP(), g); }

BOOST_SHIM_T std::pair<shim_edge_descriptor, bool> add_edge(shim_vertex_descriptor u, shim_vertex_descriptor v,
                                                            const EP& p, BOOST_SHIM_G& g) {
    typedef typename BOOST_SHIM_G::vnode VN;
    auto* e = new typename BOOST_SHIM_G::enode();
    e->prop = p;
    e->s = static_cast<VN*>(u.p);
    e->t = static_cast<VN*>(v.p);
    e->at_out = e->s->out.insert(e->s->out.end(), e);
    e->at_in = e->t->in.insert(e->t->in.end(), e);
    e->at = g.elist.insert(g.elist.end(), e);
    return {shim_edge_descriptor(e), true};
}
BOOST_SHIM_T std::pair<shim_edge_descriptor, bool> add_edge(shim_vertex_descriptor u, shim_vertex_descriptor v,
                                                            BOOST_SHIM_G& g) {
    return add_edge(u, v, EP(), g);
}

BOOST_SHIM_T shim_vertex_descriptor source(shim_edge_descriptor e, const BOOST_SHIM_G&) {
    return shim_vertex_descriptor(static_cast<typename BOOST_SHIM_G::enode*>(e.p)->s);
}
BOOST_SHIM_T shim_vertex_descriptor target(shim_edge_descriptor e, const BOOST_SHIM_G&) {
    return shim_vertex_descriptor(static_cast<typename BOOST_SHIM_G::enode*>(e.p)->t);
}

BOOST_SHIM_T std::pair<typename BOOST_SHIM_G::vertex_iterator, typename BOOST_SHIM_G::vertex_iterator> vertices(
    const BOOST_SHIM_G& g) {
    typedef typename BOOST_SHIM_G::vertex_iterator It;
    return {It(g.vlist.cbegin()), It(g.vlist.cend())};
}
BOOST_SHIM_T std::pair<typename BOOST_SHIM_G::edge_iterator, typename BOOST_SHIM_G::edge_iterator> edges(
    const BOOST_SHIM_G& g) {
    typedef typename BOOST_SHIM_G::edge_iterator It;
    return {It(g.elist.cbegin()), It(g.elist.cend())};
}
BOOST_SHIM_T std::pair<typename BOOST_SHIM_G::out_edge_iterator, typename BOOST_SHIM_G::out_edge_iterator> out_edges(
    shim_vertex_descriptor v, const BOOST_SHIM_G&) {
    typedef typename BOOST_SHIM_G::out_edge_iterator It;
    const auto* n = static_cast<const typename BOOST_SHIM_G::vnode*>(v.p);
    return {It(n->out.cbegin()), It(n->out.cend())};
}
BOOST_SHIM_T std::pair<typename BOOST_SHIM_G::in_edge_iterator, typename BOOST_SHIM_G::in_edge_iterator> in_edges(
    shim_vertex_descriptor v, const BOOST_SHIM_G&) {
    typedef typename BOOST_SHIM_G::in_edge_iterator It;
    const auto* n = static_cast<const typename BOOST_SHIM_G::vnode*>(v.p);
    return {It(n->in.cbegin()), It(n->in.cend())};
}
BOOST_SHIM_T std::size_t out_degree(shim_vertex_descriptor v, const BOOST_SHIM_G&) {
    return static_cast<const typename BOOST_SHIM_G::vnode*>(v.p)->out.size();
}
BOOST_SHIM_T std::size_t in_degree(shim_vertex_descriptor v, const BOOST_SHIM_G&) {
    return static_cast<const typename BOOST_SHIM_G::vnode*>(v.p)->in.size();
}
// bidirectional graphs: out-degree plus in-degree
BOOST_SHIM_T std::size_t degree(shim_vertex_descriptor v, const BOOST_SHIM_G& g) {
    return out_degree(v, g) + in_degree(v, g);
}
BOOST_SHIM_T std::size_t num_vertices(const BOOST_SHIM_G& g) { return g.vlist.size(); }
BOOST_SHIM_T std::size_t num_edges(const BOOST_SHIM_G& g) { return g.elist.size(); }

// the first edge u -> v in u's out-edge order
BOOST_SHIM_T std::pair<shim_edge_descriptor, bool> edge(shim_vertex_descriptor u, shim_vertex_descriptor v,
                                                        const BOOST_SHIM_G&) {
    const auto* n = static_cast<const typename BOOST_SHIM_G::vnode*>(u.p);
    for (auto* e : n->out)
        if (e->t == v.p) return {shim_edge_descriptor(e), true};
    return {shim_edge_descriptor(), false};
}

BOOST_SHIM_T void remove_edge(shim_edge_descriptor ed, BOOST_SHIM_G& g) {
    auto* e = static_cast<typename BOOST_SHIM_G::enode*>(ed.p);
    e->s->out.erase(e->at_out);
    e->t->in.erase(e->at_in);
    g.elist.erase(e->at);
    delete e;
}
// every edge u -> v
BOOST_SHIM_T void remove_edge(shim_vertex_descriptor u, shim_vertex_descriptor v, BOOST_SHIM_G& g) {
    auto* n = static_cast<typename BOOST_SHIM_G::vnode*>(u.p);
    std::vector<typename BOOST_SHIM_G::enode*> gone;
    for (auto* e : n->out)
        if (e->t == v.p) gone.push_back(e);
    for (auto* e : gone) remove_edge(shim_edge_descriptor(e), g);
}
BOOST_SHIM_T void clear_vertex(shim_vertex_descriptor v, BOOST_SHIM_G& g) {
    auto* n = static_cast<typename BOOST_SHIM_G::vnode*>(v.p);
    while (!n->out.empty()) remove_edge(shim_edge_descriptor(n->out.front()), g);
    while (!n->in.empty()) remove_edge(shim_edge_descriptor(n->in.front()), g);
}
BOOST_SHIM_T void remove_vertex(shim_vertex_descriptor v, BOOST_SHIM_G& g) {
    auto* n = static_cast<typename BOOST_SHIM_G::vnode*>(v.p);
    g.vlist.erase(n->at);
    delete n;
}

#undef BOOST_SHIM_G
#undef BOOST_SHIM_T

using std::tie;

}  // namespace boost
