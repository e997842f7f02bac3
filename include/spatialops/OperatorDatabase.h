// OperatorDatabase: a registry of operator objects keyed by their C++ type, each type holding
// any number of instances by integer id (drop-in for spatialops/OperatorDatabase.h:56-253: same
// retrieval rules and error behaviour -- id -1 means "the only one", several registered
// instances need an explicit id, a missing type or id throws std::runtime_error).
#ifndef SpatialOps_OperatorDatabase_h
#define SpatialOps_OperatorDatabase_h

#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <typeindex>
#include <typeinfo>

namespace SpatialOps {

class OperatorDatabase {
  struct StoreBase {
    virtual ~StoreBase() {}
  };
  template <typename OpT>
  struct OpStore : StoreBase {
    std::map<int, std::unique_ptr<OpT>> ops;
    int counter = 0;
    int add(OpT* op) {
      ops[++counter].reset(op);
      return counter;
    }
    OpT* get(int id) const {
      auto it = ops.begin();
      if (id == -1) {
        if (ops.size() > 1) {
          std::ostringstream msg;
          msg << "ERROR!  You must provide a unique identifier, since multiple operators have been registered."
              << std::endl
              << "        registered ids:" << std::endl;
          for (auto& kv : ops) msg << "     " << kv.first << std::endl;
          throw std::runtime_error(msg.str());
        }
      } else {
        it = ops.find(id);
      }
      if (it == ops.end()) {
        std::ostringstream msg;
        msg << "ERROR!  Attempted to retrieve an operator that does not exist." << std::endl
            << "        Operator type name: " << typeid(OpT).name() << std::endl
            << "   Registered ids:" << std::endl;
        for (auto& kv : ops) msg << "     " << kv.first << std::endl;
        throw std::runtime_error(msg.str());
      }
      return it->second.get();
    }
  };
  std::map<std::type_index, std::unique_ptr<StoreBase>> stores_;

  template <typename OpT>
  OpStore<OpT>* find() const {
    auto it = stores_.find(std::type_index(typeid(OpT)));
    return it == stores_.end() ? nullptr : static_cast<OpStore<OpT>*>(it->second.get());
  }

 public:
  OperatorDatabase() {}
  OperatorDatabase(const OperatorDatabase&) = delete;
  OperatorDatabase& operator=(const OperatorDatabase&) = delete;

  // Takes ownership of op; returns its id within its type.
  template <typename OpT>
  int register_new_operator(OpT* const op) {
    OpStore<OpT>* s = find<OpT>();
    if (!s) {
      s = new OpStore<OpT>();
      stores_[std::type_index(typeid(OpT))].reset(s);
    }
    return s->add(op);
  }

  template <typename OpT>
  OpT* retrieve_operator(const int id = -1) const {
    const OpStore<OpT>* s = find<OpT>();
    if (!s) {
      std::ostringstream msg;
      msg << "ERROR!  Attempted to retrieve an operator that does not exist." << std::endl
          << "        Operator type name: " << typeid(OpT).name() << std::endl;
      throw std::runtime_error(msg.str());
    }
    return s->get(id);
  }

  void empty_database() { stores_.clear(); }
};

}  // namespace SpatialOps
#endif
