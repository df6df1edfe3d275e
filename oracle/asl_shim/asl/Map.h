// From-scratch stand-in for asl/Map.h (see defs.h): an ordered map; Dic is a
// map keyed by String.  Iteration yields entries with .key and .value in key
// order.
#ifndef ASL_SHIM_MAP_H
#define ASL_SHIM_MAP_H
#include "defs.h"
#include "String.h"
#include <map>
namespace asl {
template <class K, class V>
class Map {
 public:
  struct Entry {
    K key;
    V value;
  };

 private:
  std::map<K, Entry> m_;

 public:
  V& operator[](const K& k) {
    auto it = m_.find(k);
    if (it == m_.end()) it = m_.emplace(k, Entry{k, V()}).first;
    return it->second.value;
  }
  bool has(const K& k) const { return m_.count(k) != 0; }
  V get(const K& k, const V& def) const {
    auto it = m_.find(k);
    return it == m_.end() ? def : it->second.value;
  }
  int length() const { return (int)m_.size(); }
  struct iterator {
    typename std::map<K, Entry>::iterator it;
    Entry& operator*() const { return it->second; }
    iterator& operator++() { ++it; return *this; }
    bool operator!=(const iterator& o) const { return it != o.it; }
  };
  iterator begin() { return iterator{m_.begin()}; }
  iterator end() { return iterator{m_.end()}; }
};
template <class V>
using Dic = Map<String, V>;
}  // namespace asl
#endif
