// Declaration-only stand-in for the yaml-cpp API the reference's headers name, so the
// GPU gate can be syntax-checked against those headers where yaml-cpp is not installed.
// Nothing here is ever linked or run.
#pragma once
#include <cstddef>
#include <string>
#include <vector>

namespace YAML {
struct NodeType {
    enum value { Undefined, Null, Scalar, Sequence, Map };
};
class Node;
class iterator {
  public:
    Node operator*() const;
    const Node* operator->() const;
    iterator& operator++();
    bool operator!=(const iterator&) const;
    bool operator==(const iterator&) const;
};
class Node {
  public:
    Node();
    Node(const Node&);
    template <class T> explicit Node(const T&);
    Node& operator=(const Node&);
    template <class T> Node& operator=(const T&);
    bool IsDefined() const;
    bool IsNull() const;
    bool IsScalar() const;
    bool IsSequence() const;
    bool IsMap() const;
    explicit operator bool() const;
    bool operator!() const;
    std::size_t size() const;
    const std::string& Scalar() const;
    const std::string& Tag() const;
    template <class T> T as() const;
    template <class T, class S> T as(const S&) const;
    Node operator[](std::size_t) const;
    Node operator[](std::size_t);
    Node operator[](const std::string&) const;
    Node operator[](const std::string&);
    Node operator[](const char*) const;
    Node operator[](const char*);
    Node operator[](const Node&) const;
    template <class T> void push_back(const T&);
    bool remove(const std::string&);
    NodeType::value Type() const;
    iterator begin() const;
    iterator end() const;
};
Node Load(const std::string&);
Node LoadFile(const std::string&);
class Emitter {
  public:
    Emitter();
    const char* c_str() const;
    template <class T> Emitter& operator<<(const T&);
};
}  // namespace YAML
