// cujson_iter.h -- query iterators over a parse result, with the reference's
// class and method names and navigation rules:
//   cuJSONIterator       <- cujson/query/query_iterator_standard_json.cpp:22-573
//   cuJSONLinesIterator  <- cujson/query/query_iterator.cpp:21-629
//
// An iterator re-reads the JSON file, walks structural[] (byte positions of
// { } [ ] : , and of newlines in JSON Lines) and jumps over containers with
// pair_pos[].  The node index is an index into structural[]; node 0 is the
// virtual root '[' and node S+1 the virtual ']'.
//
// The navigation steps keep the reference's exact rules, including its
// quirks (a ',' seen through getChar is what the reference compares against
// '\n'; the JSON-Lines iterator also counts ' ' as an element separator in
// gotoArrayIndex), so that queries answer the same on the same result.  Where
// the reference reads outside the file or the result (getChar of the virtual
// root, negative lengths) this version checks bounds; getKey on a node that is
// not a ':' returns "" instead of exiting the process.
#ifndef CUJSON_ITER_H
#define CUJSON_ITER_H

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "../cujson_gb300.h"
#include "cujson_types.h"

namespace cujson_detail {

// Shared navigation; `lines` selects the JSON-Lines variants of the rules.
class IteratorBase {
public:
    uint8_t* inputJSON = nullptr;
    std::vector<int> resultSizes;
    std::vector<int> resultSizesPrefix;
    int32_t* structural = nullptr;
    int32_t* pair_pos = nullptr;
    int jsonDepth = 0;
    int bufferSize = 0;
    int totalResultSize = 0;
    int chunkCount = 0;
    int currentChunkIndex = 0;
    int fileSize = 0;
    token_type nodeType = OBJECT;
    int node = 0;
    size_t len = 0;

    IteratorBase(cuJSONResult* parsedTree, const char* filePath, bool lines) : lines_(lines)
    {
        if (!readFile(filePath, inputJSON, len))
            std::cout << "Failed to Open File for Query!\n";
        resultSizes = parsedTree->resultSizes;
        resultSizesPrefix = parsedTree->resultSizesPrefix;
        totalResultSize = parsedTree->totalResultSize;
        structural = parsedTree->structural;
        fileSize = parsedTree->fileSize;
        pair_pos = parsedTree->pair_pos;
        if (structural && totalResultSize >= 2) {
            structural[0] = 0;
            structural[totalResultSize - 1] = fileSize - 1;
            pair_pos[0] = totalResultSize - 1;
        }
        jsonDepth = parsedTree->depth;
        bufferSize = parsedTree->bufferSize;
        chunkCount = parsedTree->chunkCount;
        currentChunkIndex = 0;
    }

    // byte of the file at a 0-based position, 0 outside the file
    uint8_t at(long pos) const { return (pos >= 0 && (size_t)pos < len) ? inputJSON[pos] : 0; }

    char getChar(int idx) const
    {
        if (idx < 0 || idx >= totalResultSize) return '\0';
        if (at((long)structural[idx] - 1) == '\n') return ',';
        if (idx == totalResultSize - 1) return ']';
        if (idx == 0) return '[';
        return (char)at((long)structural[idx] - 1);
    }

    char getArtificalChar(int idx) const { return idx == totalResultSize - 1 ? ']' : '\0'; }

    int jumpOpeningForward(int idx) const
    {
        return (idx >= 0 && idx < totalResultSize) ? pair_pos[idx] : idx;
    }

    int jumpSpacesForward(int pos) const
    {
        while (at(pos) == ' ') pos++;
        return pos;
    }

    int jumpSpacesBackward(int pos) const
    {
        while (pos >= 0 && at(pos) == ' ') pos--;
        return pos;
    }

    int jumpValueBackward(int pos) const
    {
        int cur = pos - 1;
        while (cur >= 0 && (at(cur) == ' ' || at(cur) == '"')) {
            if (at(cur) == '"') return cur - 1;
            cur--;
        }
        return cur;
    }

    int jumpValueForward(int pos) const
    {
        int cur = pos + 1;
        while (at(cur) == ' ' || at(cur) == '"') {
            if (at(cur) == '"') return cur + 1;
            cur++;
        }
        return cur;
    }

    int jumpForwardStructural(int idx) const
    {
        int cur = idx + 1;
        char c = getChar(cur);
        while (cur < totalResultSize && (c == '}' || c == ']' || c == getArtificalChar(cur))) {
            cur++;
            c = getChar(cur);
        }
        return cur;
    }

    bool readFile(const char* file, uint8_t*& buffer, size_t& size)
    {
        FILE* h = file ? fopen(file, "rb") : nullptr;
        if (!h) {
            std::cerr << "File not found!" << std::endl;
            return false;
        }
        fseek(h, 0, SEEK_END);
        long n = ftell(h);
        fseek(h, 0, SEEK_SET);
        if (n < 0) { fclose(h); return false; }
        buffer = static_cast<uint8_t*>(malloc(n > 0 ? (size_t)n : 1));
        if (!buffer) { fclose(h); return false; }
        size = (size_t)n;
        if (fread(buffer, 1, size, h) != size) {
            free(buffer);
            buffer = nullptr;
            size = 0;
            fclose(h);
            return false;
        }
        fclose(h);
        return true;
    }

    void reset()
    {
        node = 0;
        currArrayNode_ = 0;
        nodeType = OBJECT;
    }

    void freeJson()
    {
        free(inputJSON);
        inputJSON = nullptr;
        cj_host_free(structural);
        structural = nullptr;
        pair_pos = nullptr;
    }

    int increamentIndex(int index)
    {
        node = node + index;
        const char c = getChar(node);
        if (c == '{') nodeType = OBJECT;
        else if (c == '[') nodeType = ARRAY;
        else if (c == ',' || c == '\n') nodeType = VALUE;
        else if (c == ':') nodeType = KEYVALUE;
        else if (c == ']' || c == '}') nodeType = CLOSING;
        else return 0;
        return node;
    }

    // shared by gotoArrayIndex and the JSON-Lines sibling helper
    int walkArray(int index, bool step_from_separator, bool sibling)
    {
        int total = index + 1;
        const char currentNodeChar = getChar(node);
        if (step_from_separator &&
            (currentNodeChar == ',' || currentNodeChar == '\n' || currentNodeChar == ':'))
            increamentIndex(1);
        int nextNode = node + 1;
        char nextNodeChar = getChar(nextNode);
        while (total != 1 && nextNodeChar != ']' && nextNode < totalResultSize - 1) {
            if (nextNodeChar == '[' || nextNodeChar == '{') nextNode = jumpOpeningForward(nextNode);
            if (nextNodeChar == ',' || nextNodeChar == '\n' || (lines_ && nextNodeChar == ' ')) {
                if (lines_ && !sibling) currArrayNode_ = nextNode;
                total--;
            }
            nextNode++;
            nextNodeChar = getChar(nextNode);
        }
        if (total != 1) return 0;
        node = nextNode - 1;
        if (sibling) currArrayNode_ = node;
        if (nextNodeChar == '{') {
            nodeType = OBJECT;
        } else if (nextNodeChar == '[') {
            nodeType = ARRAY;
            if (!lines_) {
                node = nextNode;
                return node;
            }
        } else if (nextNodeChar == ',' || currentNodeChar == '\n' || nextNodeChar == ']') {
            nodeType = VALUE;
        }
        return node;
    }

    int gotoArrayIndex(int index) { return walkArray(index, true, false); }

    std::string getString(int startPos, int endPos) const
    {
        startPos = jumpSpacesForward(startPos + 1);
        endPos = jumpSpacesBackward(endPos - 1);
        const int length = std::abs(endPos - startPos - 1);
        return slice(startPos + 1, length);
    }

    int findKey(const std::string& input_key)
    {
        char currentNodeChar = getChar(node);
        int nextNode = node;
        if (currentNodeChar == ':' || currentNodeChar == ',' || currentNodeChar == '\n') nextNode = nextNode + 1;
        const char nextPossibleNodeChar = getChar(node + 1);
        if (currentNodeChar == '[' && nextPossibleNodeChar == '{') nextNode = node + 1;
        if (getChar(nextNode) != '{') {
            if (!lines_) std::cout << "ERROR: Node is not an object to find key!" << std::endl;
            return 0;
        }
        const int endNode = jumpOpeningForward(nextNode);
        nextNode = nextNode + 1;
        char nextNodeChar = getChar(nextNode);
        while (nextNode < endNode && nextNodeChar != '}') {
            if (nextNodeChar == '[' || nextNodeChar == '{') nextNode = jumpOpeningForward(nextNode);
            if (nextNodeChar == ':') {
                const int endPos = structural[nextNode] - 1;
                const int startPos = structural[nextNode - 1] - 1;
                if (getString(startPos, endPos) == input_key) return nextNode - node;
            }
            nextNode++;
            nextNodeChar = getChar(nextNode);
        }
        return 0;
    }

    int gotoKey(const std::string& key) { return increamentIndex(findKey(key)); }

    std::string getKey() const
    {
        if (getChar(node) != ':') {
            std::cout << "ERROR! The iterator must point to a colon.";
            return std::string();
        }
        return getString(structural[node - 1] - 1, structural[node] - 1);
    }

    std::string getValue() const
    {
        const char c = getChar(node);
        if (c != ',' && c != '\n' && c != ':' && c != '[') {
            std::cout << "ERROR: iterator is in wrong place." << std::endl;
            return std::string();
        }
        int startIdx = node + 1;
        const char nextNodeChar = getChar(startIdx);
        int startPos, endPos;
        if (nextNodeChar == '[' || nextNodeChar == '{') {
            const int endIdx = jumpOpeningForward(startIdx);
            startPos = structural[startIdx] - 1;
            endPos = structural[endIdx] - 1;
        } else {
            const int endIdx = startIdx;
            startIdx = node;
            startPos = jumpValueForward(structural[startIdx] - 1);
            endPos = jumpValueBackward(structural[endIdx] - 1);
        }
        return slice(startPos, endPos - startPos + 1);
    }

protected:
    std::string slice(long start, long length) const
    {
        if (length <= 0 || start < 0 || (size_t)start >= len) return std::string();
        if ((size_t)(start + length) > len) length = (long)len - start;
        return std::string(reinterpret_cast<const char*>(inputJSON) + start, (size_t)length);
    }

    bool lines_;
    int currArrayNode_ = 0;
};

}  // namespace cujson_detail

class cuJSONIterator : public cujson_detail::IteratorBase {
public:
    cuJSONIterator(cuJSONResult* parsedTree, const char* filePath)
        : IteratorBase(parsedTree, filePath, false) {}
};

class cuJSONLinesIterator : public cujson_detail::IteratorBase {
public:
    cuJSONLinesIterator(cuJSONResult* parsedTree, const char* filePath)
        : IteratorBase(parsedTree, filePath, true) {}

    int gotoArrayIndexSiblingHelper(int index) { return walkArray(index, false, true); }

    int gotoNextSibling(int index)
    {
        node = currArrayNode_;
        return gotoArrayIndexSiblingHelper(index);
    }

    bool checkKeyValue(const std::string& key, const std::string& value)
    {
        const int index1 = findKey(key);
        if (index1 == 0) return false;
        const int currentNode = node;
        increamentIndex(index1);
        const std::string currentValue = getValue();
        node = currentNode;
        return currentValue == value;
    }
};

#endif  // CUJSON_ITER_H
