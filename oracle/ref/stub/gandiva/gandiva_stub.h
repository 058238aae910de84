/*
 * Oracle build shim (test infrastructure only).
 *
 * The reference Splitter (native-sql-engine/cpp/src/shuffle/splitter.{h,cc}) asks gandiva
 * to JIT the partition hash chain (splitter.cc:1402-1447).  gandiva is not available here,
 * and the hash bodies live in the un-vendored Arrow fork, so this header provides the few
 * gandiva names the Splitter uses (ExpressionVector, TreeExprBuilder, Projector) with an
 * interpreter that evaluates the same chain with the restated Spark Murmur3 from
 * oracle/spark_hash.h.  Everything after the projector (pmod, histogram, scatter, buffer
 * policy, IPC) is the reference's own code, compiled unchanged from its source tree.
 */
#pragma once

#include <arrow/api.h>

#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../../spark_hash.h"

namespace gandiva {

class Node;
using NodePtr = std::shared_ptr<Node>;
using NodeVector = std::vector<NodePtr>;
using FieldVector = std::vector<std::shared_ptr<arrow::Field>>;
using DataTypePtr = std::shared_ptr<arrow::DataType>;

class Node {
 public:
  enum Kind { kField, kLiteral, kFunction };
  Node(Kind k, DataTypePtr t) : kind_(k), type_(std::move(t)) {}
  virtual ~Node() = default;
  const DataTypePtr& return_type() const { return type_; }
  Kind kind() const { return kind_; }

  std::shared_ptr<arrow::Field> field;  // kField
  int32_t literal = 0;                  // kLiteral
  std::string name;                     // kFunction
  NodeVector children;                  // kFunction

 private:
  Kind kind_;
  DataTypePtr type_;
};

class Expression {
 public:
  Expression(NodePtr root, std::shared_ptr<arrow::Field> result)
      : root_(std::move(root)), result_(std::move(result)) {}
  const NodePtr& root() const { return root_; }
  const std::shared_ptr<arrow::Field>& result() const { return result_; }

 private:
  NodePtr root_;
  std::shared_ptr<arrow::Field> result_;
};
using ExpressionPtr = std::shared_ptr<Expression>;
using ExpressionVector = std::vector<ExpressionPtr>;

class TreeExprBuilder {
 public:
  static NodePtr MakeLiteral(int32_t v) {
    auto n = std::make_shared<Node>(Node::kLiteral, arrow::int32());
    n->literal = v;
    return n;
  }
  static NodePtr MakeField(std::shared_ptr<arrow::Field> f) {
    auto n = std::make_shared<Node>(Node::kField, f->type());
    n->field = std::move(f);
    return n;
  }
  static NodePtr MakeFunction(const std::string& name, const NodeVector& params,
                              DataTypePtr ret) {
    auto n = std::make_shared<Node>(Node::kFunction, std::move(ret));
    n->name = name;
    n->children = params;
    return n;
  }
  static ExpressionPtr MakeExpression(NodePtr root, std::shared_ptr<arrow::Field> result) {
    return std::make_shared<Expression>(std::move(root), std::move(result));
  }
};

namespace stub_internal {

inline bool BitIsSet(const uint8_t* bits, int64_t i) { return (bits[i >> 3] >> (i & 7)) & 1; }

// Spark UTF8String.hashUnsafeBytes: 4-byte blocks, then every tail byte mixed as its own
// sign-extended int; length = byte count.
inline int32_t SparkHashBytes(const uint8_t* p, int32_t len, int32_t seed) {
  using namespace gzoracle;
  uint32_t h1 = (uint32_t)seed;
  int32_t aligned = len - len % 4;
  for (int32_t i = 0; i < aligned; i += 4) {
    uint32_t k;
    memcpy(&k, p + i, 4);
    h1 = mix_h1(h1, mix_k1(k));
  }
  for (int32_t i = aligned; i < len; i++) {
    int32_t half = (int8_t)p[i];
    h1 = mix_h1(h1, mix_k1((uint32_t)half));
  }
  return (int32_t)fmix32(h1, (uint32_t)len);
}

// One value of a key column hashed into `seed`; nulls pass the seed through.
inline arrow::Status HashValue(const std::string& fn, const arrow::ArrayData& a, int64_t row,
                               int32_t seed, int32_t* out) {
  using namespace gzoracle;
  const uint8_t* valid = a.buffers[0] ? a.buffers[0]->data() : nullptr;
  if (valid != nullptr && a.buffers[0]->size() > 0 && !BitIsSet(valid, row + a.offset)) {
    *out = seed;
    return arrow::Status::OK();
  }
  const uint8_t* v = a.buffers.size() > 1 && a.buffers[1] ? a.buffers[1]->data() : nullptr;
  int64_t i = row + a.offset;
  switch (a.type->id()) {
    case arrow::Type::BOOL:
      *out = spark_hash_int(BitIsSet(v, i) ? 1 : 0, seed);
      break;
    case arrow::Type::INT8:
      *out = spark_hash_int(reinterpret_cast<const int8_t*>(v)[i], seed);
      break;
    case arrow::Type::INT16:
      *out = spark_hash_int(reinterpret_cast<const int16_t*>(v)[i], seed);
      break;
    case arrow::Type::INT32:
    case arrow::Type::DATE32:
    case arrow::Type::FLOAT:
      *out = spark_hash_int(reinterpret_cast<const int32_t*>(v)[i], seed);
      break;
    case arrow::Type::INT64:
    case arrow::Type::DOUBLE:
      *out = spark_hash_long(reinterpret_cast<const int64_t*>(v)[i], seed);
      break;
    case arrow::Type::STRING: {
      const int32_t* off = reinterpret_cast<const int32_t*>(v);
      const uint8_t* chars = a.buffers[2] ? a.buffers[2]->data() : nullptr;
      *out = SparkHashBytes(chars + off[i], off[i + 1] - off[i], seed);
      break;
    }
    default:
      return arrow::Status::NotImplemented("hash of type ", a.type->ToString(),
                                           " is not available in the oracle build");
  }
  (void)fn;
  return arrow::Status::OK();
}

inline arrow::Status Eval(const Node& n, const arrow::RecordBatch& rb, int64_t row,
                          int32_t* out) {
  switch (n.kind()) {
    case Node::kLiteral:
      *out = n.literal;
      return arrow::Status::OK();
    case Node::kField:
      return arrow::Status::Invalid("bare field in hash chain");
    case Node::kFunction: {
      if (n.name != "hash32_spark" && n.name != "hash64_spark" && n.name != "hashbuf_spark") {
        return arrow::Status::NotImplemented("function ", n.name,
                                             " is not available in the oracle build");
      }
      int32_t seed;
      ARROW_RETURN_NOT_OK(Eval(*n.children[1], rb, row, &seed));
      const Node& key = *n.children[0];
      if (key.kind() != Node::kField) {
        return arrow::Status::NotImplemented("only field references are hashed");
      }
      int idx = rb.schema()->GetFieldIndex(key.field->name());
      if (idx < 0) return arrow::Status::Invalid("unknown key field ", key.field->name());
      return HashValue(n.name, *rb.column_data(idx), row, seed, out);
    }
  }
  return arrow::Status::Invalid("bad node");
}

}  // namespace stub_internal

class Projector {
 public:
  static arrow::Status Make(std::shared_ptr<arrow::Schema> schema, const ExpressionVector& exprs,
                            std::shared_ptr<Projector>* out) {
    for (const auto& e : exprs) {
      ARROW_RETURN_NOT_OK(Check(*e->root()));
    }
    auto p = std::make_shared<Projector>();
    p->schema_ = std::move(schema);
    p->exprs_ = exprs;
    *out = std::move(p);
    return arrow::Status::OK();
  }

  arrow::Status Evaluate(const arrow::RecordBatch& rb, arrow::MemoryPool* pool,
                         arrow::ArrayVector* outputs) const {
    for (const auto& e : exprs_) {
      arrow::Int32Builder b(pool);
      ARROW_RETURN_NOT_OK(b.Reserve(rb.num_rows()));
      for (int64_t r = 0; r < rb.num_rows(); ++r) {
        int32_t h;
        ARROW_RETURN_NOT_OK(stub_internal::Eval(*e->root(), rb, r, &h));
        b.UnsafeAppend(h);
      }
      std::shared_ptr<arrow::Array> arr;
      ARROW_RETURN_NOT_OK(b.Finish(&arr));
      outputs->push_back(std::move(arr));
    }
    return arrow::Status::OK();
  }

 private:
  static arrow::Status Check(const Node& n) {
    if (n.kind() == Node::kFunction) {
      if (n.name != "hash32_spark" && n.name != "hash64_spark" && n.name != "hashbuf_spark") {
        return arrow::Status::NotImplemented("function ", n.name,
                                             " is not available in the oracle build");
      }
      for (const auto& c : n.children) ARROW_RETURN_NOT_OK(Check(*c));
    }
    return arrow::Status::OK();
  }
  std::shared_ptr<arrow::Schema> schema_;
  ExpressionVector exprs_;
};

}  // namespace gandiva
