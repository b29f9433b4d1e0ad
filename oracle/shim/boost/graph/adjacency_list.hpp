// Declarations-only stand-in for the parts of Boost.Graph that the
// reference's interval/fiber headers name.  No graph algorithm is provided:
// the weave is not part of the oracle.  Project-written.
#pragma once
#include <list>
#include <set>
#include <tuple>
#include <utility>
#include <vector>
#include <iostream>
namespace boost {
struct listS {};
struct vecS {};
struct bidirectionalS {};
struct directedS {};
struct no_property {};
template <class A = void, class B = void, class C = void, class D = void>
struct adjacency_list_traits {
    typedef void* vertex_descriptor;
    typedef void* edge_descriptor;
};
template <class A = void, class B = void, class C = void, class D = void,
          class E = void, class F = void, class G = void>
struct adjacency_list {
    typedef void* vertex_descriptor;
    typedef void* edge_descriptor;
};
template <class G> struct graph_traits {
    typedef void* vertex_descriptor;
    typedef void* edge_descriptor;
    typedef void** vertex_iterator;
    typedef void** edge_iterator;
    typedef void** out_edge_iterator;
    typedef void** adjacency_iterator;
    typedef unsigned long vertices_size_type;
    typedef unsigned long edges_size_type;
    typedef unsigned long degree_size_type;
    static vertex_descriptor null_vertex() { return nullptr; }
};
template <class... T> void* add_vertex(T&&...) { return nullptr; }
template <class... T> std::pair<void*, bool> add_edge(T&&...) { return {nullptr, false}; }
template <class... T> void clear_vertex(T&&...) {}
template <class... T> void remove_vertex(T&&...) {}
template <class... T> void remove_edge(T&&...) {}
template <class... T> unsigned long degree(T&&...) { return 0; }
template <class... T> std::pair<void*, bool> edge(T&&...) { return {nullptr, false}; }
template <class... T> std::pair<void**, void**> edges(T&&...) { return {nullptr, nullptr}; }
template <class... T> std::pair<void**, void**> vertices(T&&...) { return {nullptr, nullptr}; }
template <class... T> std::pair<void**, void**> out_edges(T&&...) { return {nullptr, nullptr}; }
template <class... T> unsigned long num_edges(T&&...) { return 0; }
template <class... T> unsigned long num_vertices(T&&...) { return 0; }
template <class... T> void* source(T&&...) { return nullptr; }
template <class... T> void* target(T&&...) { return nullptr; }
using std::tie;
}
