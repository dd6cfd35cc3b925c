// Stand-in for the part of rapidjson's DOM that Neon's Report classes use.
// Values and documents accept every member and discard it: the reports the
// reference writes are not needed to run its hot path.
#pragma once
#include <cstdint>
#include <string>

namespace rapidjson {
using SizeType = unsigned;
enum Type { kNullType = 0, kFalseType, kTrueType, kObjectType, kArrayType, kStringType, kNumberType };

struct MemoryPoolAllocator {
};

class Value
{
   public:
    Value() = default;
    explicit Value(Type) {}
    Value(const char*, MemoryPoolAllocator&) {}
    Value(const char*, SizeType, MemoryPoolAllocator&) {}
    template <typename T>
    explicit Value(T) {}
    Value& SetInt(int) { return *this; }
    Value& SetInt64(int64_t) { return *this; }
    Value& SetUint(unsigned) { return *this; }
    Value& SetUint64(uint64_t) { return *this; }
    Value& SetDouble(double) { return *this; }
    Value& SetFloat(float) { return *this; }
    Value& SetBool(bool) { return *this; }
    Value& SetString(const char*, SizeType, MemoryPoolAllocator&) { return *this; }
    Value& SetString(const char*, SizeType) { return *this; }
    Value& SetObject() { return *this; }
    Value& SetArray() { return *this; }
    Value& Move() { return *this; }
    template <typename V, typename A>
    Value& PushBack(V&&, A&) { return *this; }
    template <typename K, typename V, typename A>
    Value& AddMember(K&&, V&&, A&) { return *this; }
};

class Document : public Value
{
   public:
    Document() = default;
    explicit Document(MemoryPoolAllocator*) {}
    MemoryPoolAllocator& GetAllocator() { return mAlloc; }
    template <typename W>
    bool Accept(W&) const { return true; }

   private:
    MemoryPoolAllocator mAlloc;
};
}  // namespace rapidjson
