// Minimal stand-in for the parts of boost::property_tree that the DROPS
// sources name.  Written for this project (no Boost source is used); it is
// only good enough to compile the reference's hot-path translation units into
// the oracle harness, which never reads a JSON parameter file.  Paths are
// dot-separated keys, data is a string, conversions go through iostreams.
#pragma once
#include <list>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>

namespace boost {
namespace property_tree {

struct ptree_error : std::runtime_error {
    explicit ptree_error(const std::string& w) : std::runtime_error(w) {}
};
struct ptree_bad_path : ptree_error {
    explicit ptree_bad_path(const std::string& w) : ptree_error(w) {}
};
struct ptree_bad_data : ptree_error {
    explicit ptree_bad_data(const std::string& w) : ptree_error(w) {}
};

class ptree {
  public:
    typedef std::string key_type;
    typedef std::string data_type;
    typedef std::string path_type;
    typedef std::pair<const std::string, ptree> value_type;
    typedef std::list<value_type> list_type;
    typedef list_type::iterator iterator;
    typedef list_type::const_iterator const_iterator;
    typedef list_type::iterator assoc_iterator;
    typedef list_type::const_iterator const_assoc_iterator;

    ptree() {}
    explicit ptree(const std::string& d) : data_(d) {}
    ptree(const ptree& o) : data_(o.data_), kids_(o.kids_) {}
    ptree& operator=(const ptree& o) {
        if (this != &o) {
            list_type tmp(o.kids_);
            data_ = o.data_;
            kids_.swap(tmp);
        }
        return *this;
    }
    bool operator==(const ptree& o) const {
        if (data_ != o.data_ || kids_.size() != o.kids_.size()) return false;
        const_iterator a = kids_.begin(), b = o.kids_.begin();
        for (; a != kids_.end(); ++a, ++b)
            if (a->first != b->first || !(a->second == b->second)) return false;
        return true;
    }
    bool operator!=(const ptree& o) const { return !(*this == o); }

    iterator begin() { return kids_.begin(); }
    iterator end() { return kids_.end(); }
    const_iterator begin() const { return kids_.begin(); }
    const_iterator end() const { return kids_.end(); }
    std::size_t size() const { return kids_.size(); }
    bool empty() const { return kids_.empty(); }

    const std::string& data() const { return data_; }
    std::string& data() { return data_; }

    iterator find(const std::string& key) {
        for (iterator it = kids_.begin(); it != kids_.end(); ++it)
            if (it->first == key) return it;
        return kids_.end();
    }
    const_iterator find(const std::string& key) const {
        for (const_iterator it = kids_.begin(); it != kids_.end(); ++it)
            if (it->first == key) return it;
        return kids_.end();
    }
    iterator not_found() { return kids_.end(); }
    const_iterator not_found() const { return kids_.end(); }

    iterator push_back(const value_type& v) { kids_.push_back(v); return --kids_.end(); }
    iterator insert(iterator where, const value_type& v) { return kids_.insert(where, v); }
    template <class It> void insert(iterator where, It first, It last) { kids_.insert(where, first, last); }

    template <class T> T get_value() const {
        std::istringstream is(data_);
        T v;
        is >> v;
        if (is.fail()) throw ptree_bad_data("conversion of '" + data_ + "' failed");
        return v;
    }

    const ptree& get_child(const std::string& path) const {
        const ptree* p = walk(path);
        if (!p) throw ptree_bad_path("no such node: " + path);
        return *p;
    }
    ptree& get_child(const std::string& path) {
        const ptree* p = walk(path);
        if (!p) throw ptree_bad_path("no such node: " + path);
        return *const_cast<ptree*>(p);
    }

    template <class T> T get(const std::string& path) const { return get_child(path).template get_value<T>(); }
    template <class T> T get(const std::string& path, const T& def) const {
        const ptree* p = walk(path);
        return p ? p->template get_value<T>() : def;
    }

    ptree& put_child(const std::string& path, const ptree& child) {
        ptree& slot = make(path);
        slot = child;
        return slot;
    }
    ptree& add_child(const std::string& path, const ptree& child) { return put_child(path, child); }

    template <class T> ptree& put(const std::string& path, const T& v) {
        std::ostringstream os;
        os.precision(17);
        os << v;
        ptree& slot = make(path);
        slot.data_ = os.str();
        return slot;
    }

  private:
    std::string data_;
    list_type kids_;

    const ptree* walk(const std::string& path) const {
        const ptree* p = this;
        std::size_t start = 0;
        while (p && start <= path.size()) {
            std::size_t dot = path.find('.', start);
            std::string key = path.substr(start, dot == std::string::npos ? std::string::npos : dot - start);
            if (key.empty()) return p;
            const_iterator it = p->find(key);
            if (it == p->kids_.end()) return 0;
            p = &it->second;
            if (dot == std::string::npos) break;
            start = dot + 1;
        }
        return p;
    }
    ptree& make(const std::string& path) {
        ptree* p = this;
        std::size_t start = 0;
        for (;;) {
            std::size_t dot = path.find('.', start);
            std::string key = path.substr(start, dot == std::string::npos ? std::string::npos : dot - start);
            iterator it = p->find(key);
            if (it == p->kids_.end()) it = p->push_back(value_type(key, ptree()));
            p = &it->second;
            if (dot == std::string::npos) return *p;
            start = dot + 1;
        }
    }
};

template <> inline std::string ptree::get_value<std::string>() const { return data_; }

}  // namespace property_tree
}  // namespace boost
